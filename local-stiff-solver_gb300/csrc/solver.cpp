// GPUHybrid-compatible orchestration on one GB300.
//
// factorize (GPUHybrid::factorize, GPUHybrid.cu:195-282):
//   values -> device, gathered into the permuted row-sliced BSR operator;
//   stiff-DOF selection on the GPU (select.cu) and host post-processing
//   (postproc.cpp); dense FP64 inverses of the stiff subdomains (stiff.cu);
//   MAS setup (mas.cu) -- in place of BoomerAMG setup (GPUHybrid.cu:357-376).
// solve (GPUHybrid::solve + pcg_solve, GPUHybrid.cu:342-399, 1413-1512):
//   device-resident FP64 PCG with the multiplicative MAS - direct - MAS
//   preconditioner (custom_mixed_precond_iter, GPUHybrid.cu:521-542);
//   iterations are captured as a CUDA graph in chunks and the host polls the
//   device stop flag once per chunk.
#include "solver.hpp"

#include "baddof.hpp"
#include "host_copy.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <sstream>
#include <tuple>

namespace lss {

void launch_pcg_rz(int64_t n, const double *r, const double *z, PcgState *st, int dot_mode, GridReduce gr,
                   cudaStream_t s);
void launch_check_finite(int64_t n, const double *v, int *flag, cudaStream_t s);

namespace {
using clk = std::chrono::steady_clock;
double secs(clk::time_point t0) { return std::chrono::duration<double>(clk::now() - t0).count(); }

const char *stop_name(int s)
{
    switch (s) {
    case STOP_RUNNING: return "running";
    case STOP_CONVERGED_REL: return "converged_rel";
    case STOP_CONVERGED_ABS: return "converged_abs";
    case STOP_ZERO_PAP: return "err_zero_sdotp";
    case STOP_NEGATIVE_ALPHA: return "err_negative_alpha";
    case STOP_SUBNORMAL_ALPHA: return "err_subnormal_alpha";
    case STOP_MAX_ITER: return "max_iterations";
    case STOP_NONFINITE: return "err_nonfinite";
    default: return "unknown";
    }
}
}  // namespace

HybridSolver::HybridSolver(const Params &p) : p_(p)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        fail(LSS_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (p_.device < 0 || p_.device >= ndev) fail(LSS_ERR_INVALID_ARGUMENT, "gb300.device out of range");
    LSS_CUDA(cudaSetDevice(p_.device));
    LSS_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    for (cudaEvent_t &e : copy_ev_) LSS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    LSS_CUDA(cudaMallocHost((void **)&h_state_, sizeof(PcgState)));
    d_state_.resize(1);
    d_partials_.resize((size_t)GRID_MAX * RED_MAX_VALUES);
    d_counter_.resize(1);
    d_counter_.zero(stream_);
    d_scalar_.resize(8);
    d_bad_.resize(1);
    gr_.partials = d_partials_.data();
    gr_.counter = d_counter_.data();
}

HybridSolver::~HybridSolver()
{
    invalidate_graph();
    if (h_state_) cudaFreeHost(h_state_);
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
    for (cudaEvent_t e : copy_ev_)
        if (e) cudaEventDestroy(e);
}

void HybridSolver::set_parameters(const char *json)
{
    Params np = parse_params(json, p_);
    if (np.device != p_.device) fail(LSS_ERR_INVALID_ARGUMENT, "the device of an existing solver cannot change");
    const bool pattern_affecting = np.block_size != p_.block_size || np.max_coarse_levels != p_.max_coarse_levels;
    const bool value_affecting = pattern_affecting || np.mixed != p_.mixed || np.do_hybrid != p_.do_hybrid ||
                                 np.select_l1 != p_.select_l1 || np.jump_threshold != p_.jump_threshold ||
                                 np.gmm_tol != p_.gmm_tol || np.max_gmm_iterations != p_.max_gmm_iterations ||
                                 np.cond_threshold != p_.cond_threshold || np.decompose != p_.decompose ||
                                 np.min_sub != p_.min_sub || np.max_sub != p_.max_sub || np.expand != p_.expand ||
                                 np.float_subdomains != p_.float_subdomains ||
                                 np.multiplicative != p_.multiplicative || np.outer_spmv != p_.outer_spmv ||
                                 np.precond_residual != p_.precond_residual ||
                                 np.mas_bf16_offdiag != p_.mas_bf16_offdiag;
    p_ = np;
    if (pattern_affecting) have_pattern_ = false;
    if (value_affecting) factorized_ = false;
    invalidate_graph();
}

std::string HybridSolver::name() const
{
    // GPUHybrid.hpp:57-67
    if (p_.do_hybrid) return p_.select_l1 ? "GPUHybrid" : "GPUAMGF";
    return "GPUAMG";
}

std::vector<int32_t> HybridSolver::selected() const
{
    std::vector<int32_t> all;
    for (const auto &s : subs_) all.insert(all.end(), s.begin(), s.end());
    std::sort(all.begin(), all.end());
    return all;
}

std::string HybridSolver::info_json() const
{
    std::ostringstream o;
    o.precision(17);
    o << "{\"num_iterations\": " << num_iterations_ << ", \"final_res_norm\": " << final_res_norm_;
    o << ", \"relative_residual\": " << (rhs_norm_ > 0 ? final_res_norm_ / rhs_norm_ : 0.0);
    o << ", \"status\": \"" << stop_name(stop_reason_) << "\"";
    o << ", \"refinements\": " << refinements_;
    o << ", \"precision\": \"" << (p_.mixed ? "mixed" : "fp64") << "\"";
    o << ", \"outer_spmv\": \"" << (df32() ? "df32" : "fp64") << "\"";
    o << ", \"composition\": \"" << (p_.multiplicative ? "multiplicative" : "additive") << "\"";
    o << ", \"mas_omega\": " << omega_;
    o << ", \"kernel_launches\": " << launch_count().load();
    int64_t nstiff = 0;
    for (const auto &s : subs_) nstiff += (int64_t)s.size();
    o << ", \"num_stiff_dofs\": " << nstiff << ", \"num_subdomains\": " << subs_.size();
    o << ", \"num_gmm_selected\": " << gmm_sel_.size();
    if (have_pattern_) {
        o << ", \"num_parts\": " << (pat_.part.part_offsets.size() - 1) << ", \"mas_levels\": " << cs_.L;
        o << ", \"block_size\": " << pat_.bd << ", \"nnz_blocks\": " << pat_.rows.back();
        o << ", \"spmv_lanes\": " << A_.lanes << ", \"spmv_lanes_fp32\": " << A_.lanes32;
    }
    for (const auto &kv : stats_) o << ", \"" << kv.first << "\": " << kv.second;
    for (const auto &kv : sstats_) o << ", \"" << kv.first << "\": \"" << kv.second << "\"";
    o << "}";
    return o.str();
}

void HybridSolver::invalidate_graph()
{
    if (graph_exec_) {
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
    graph_iters_ = 0;
}

// ------------------------------------------------------------------ pattern

void HybridSolver::analyze(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner)
{
    if (!outer || !inner || n <= 0 || nnz < 0) fail(LSS_ERR_INVALID_ARGUMENT, "invalid matrix arguments");
    auto t0 = clk::now();
    invalidate_graph();
    factorized_ = false;
    have_pattern_ = false;
    // a new pattern: nothing of the previous pattern's stiff layout is reusable
    decomp_sel_.clear();
    decomp_max_ = -1;
    decomp_subs_.clear();
    h_sdofs_.clear();
    h_soff_.assign(1, 0);
    mf_.reset();
    pat_ = analyze_pattern(n, nnz, outer, inner, p_.block_size, p_.partition_threads);
    h_outer_.assign(outer, outer + n + 1);
    h_inner_.assign(inner, inner + nnz);
    d_outer_.release();
    d_inner_.release();
    d_row_of_.release();
    stats_["time_partition_and_layout"] = secs(t0);
    auto t1 = clk::now();
    cs_ = build_coarse_space(pat_, p_.max_coarse_levels);
    stats_["time_coarse_space"] = secs(t1);

    // device pattern
    d_rows_.upload(pat_.rows, stream_);
    d_cols_.upload(pat_.cols, stream_);
    d_src_.upload(pat_.src, stream_);
    d_perm_.upload(pat_.part.perm, stream_);
    d_vals_.resize(pat_.src.size());
    A_ = BsrDev();
    A_.nb = pat_.nb;
    A_.bd = pat_.bd;
    A_.rows = d_rows_.data();
    A_.cols = d_cols_.data();
    A_.vals = d_vals_.data();
    // lanes per block row: autotuned at the first factorize of this pattern
    A_.lanes = A_.lanes32 = p_.spmv_lanes > 0 ? p_.spmv_lanes : 4;
    lanes_tuned_ = p_.spmv_lanes > 0;
    // MAS device maps
    const int32_t nparts = (int32_t)pat_.part.part_offsets.size() - 1;
    d_part_off_.upload(pat_.part.part_offsets, stream_);
    d_part_of_.upload(cs_.part_of, stream_);
    d_key0_.upload(cs_.key0, stream_);
    d_ccnt0_.upload(cs_.ccnt0, stream_);
    d_cbase0_.upload(cs_.cbase0, stream_);
    d_cmap_.upload(cs_.cmap, stream_);
    d_memb_ptr_.upload(cs_.item_chunk, stream_);
    d_memb_rows_.upload(cs_.memb_rows, stream_);
    d_chunk_r0_.upload(cs_.chunk_r0, stream_);
    memb_ = CoarseMembers();
    memb_.rows = d_memb_rows_.data();
    memb_.item_chunk = d_memb_ptr_.data();
    memb_.chunk_r0 = d_chunk_r0_.data();
    memb_.nitem = (int64_t)cs_.item_chunk.size() - 1;
    memb_.nchunk = (int64_t)cs_.chunk_r0.size() - 1;
    d_key_.clear();
    d_ccnt_.clear();
    d_cbase_.clear();
    d_key_.resize(cs_.L);
    d_ccnt_.resize(cs_.L);
    d_cbase_.resize(cs_.L);
    mas_ = MasDev();
    mas_.L = cs_.L;
    mas_.bd = pat_.bd;
    mas_.nb = pat_.nb;
    mas_.nparts = nparts;
    mas_.part_off = d_part_off_.data();
    mas_.key0 = d_key0_.data();
    mas_.cbase0 = d_cbase0_.data();
    mas_.ccnt0 = d_ccnt0_.data();
    mas_.nbanks[0] = nparts;
    mas_.tile_elems = mas_tile_elems(pat_.bd);
    int64_t voff = 0;
    int32_t boff = 0;
    for (int l = 1; l < cs_.L; ++l) {
        mas_.nitems[l] = cs_.nitems[l];
        mas_.nbanks[l] = cs_.nbanks[l];
        mas_.voff[l] = voff;
        voff += (int64_t)cs_.nbanks[l] * 32 * pat_.bd;
        mas_.boff[l] = boff;
        boff += cs_.nbanks[l];
        if (l + 1 < cs_.L) {
            d_key_[l].upload(cs_.key[l], stream_);
            d_ccnt_[l].upload(cs_.ccnt[l], stream_);
            d_cbase_[l].upload(cs_.cbase[l], stream_);
            mas_.key[l] = d_key_[l].data();
            mas_.ccnt[l] = d_ccnt_[l].data();
            mas_.cbase[l] = d_cbase_[l].data();
        }
    }
    mas_.ncoarse = boff;
    mas_.level_elems = voff;
    LSS_CUDA(cudaStreamSynchronize(stream_));
    have_pattern_ = true;
    stats_["time_analyze"] = secs(t0);
    stats_["num_parts_filled_fraction"] = nparts ? (double)pat_.nb / (32.0 * nparts) : 0.0;
}

// ------------------------------------------------------------------ factorize

void HybridSolver::factorize(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                             const double *values)
{
    if (!outer || !inner || !values || n <= 0 || nnz < 0) fail(LSS_ERR_INVALID_ARGUMENT, "invalid matrix arguments");
    auto t0 = clk::now();
    factorized_ = false;
    invalidate_graph();
    // the analysed pattern is reused only if it is exactly the same (compared
    // with the stored copy on all host threads, ~10 ms for 10^8 entries)
    const int ht = host_threads();
    const bool same = have_pattern_ && pat_.n == n && pat_.nnz == nnz &&
                      parallel_equal(outer, h_outer_.data(), (size_t)(n + 1) * sizeof(int32_t), ht) &&
                      parallel_equal(inner, h_inner_.data(), (size_t)nnz * sizeof(int32_t), ht);
    stats_["time_pattern_check"] = secs(t0);
    if (!same) analyze(n, nnz, outer, inner);
    auto t1 = clk::now();
    // values -> device through pinned staging, chunks overlapped with the copies
    d_csc_.resize(nnz);
    upload_staged(d_csc_.data(), values, (size_t)nnz * sizeof(double), pin_, copy_ev_, stream_);
    factorize_common();
    stats_["time_copy_matrix_to_gpu"] = secs(t1) - stats_["time_factorize_device"];
    stats_["time_factorize"] = secs(t0);
}

void HybridSolver::factorize_device(const double *d_values, cudaStream_t user)
{
    if (!have_pattern_) fail(LSS_ERR_NOT_FACTORIZED, "factorize_device needs analyze_pattern first");
    if (!d_values) fail(LSS_ERR_INVALID_ARGUMENT, "null values");
    auto t0 = clk::now();
    factorized_ = false;
    invalidate_graph();
    StreamScope scope(this, user);
    d_csc_.resize(pat_.nnz);
    LSS_CUDA(cudaMemcpyAsync(d_csc_.data(), d_values, (size_t)pat_.nnz * sizeof(double), cudaMemcpyDeviceToDevice,
                             stream_));
    factorize_common();
    stats_["time_factorize"] = secs(t0);
}

// Everything after the values are in d_csc_: gather into the operator,
// selection, stiff factors, MAS, damping estimate.  Needs no host values.
void HybridSolver::factorize_common()
{
    auto t0 = clk::now();
    const int64_t nnz = pat_.nnz;
    d_bad_.zero(stream_);
    launch_check_finite(nnz, d_csc_.data(), d_bad_.data(), stream_);
    mas_fp32_ = p_.mixed;
    const bool df = need_vals_df();
    if (p_.mixed) d_vals32_.resize(pat_.src.size());
    else d_vals32_.release();
    if (df) d_vals_df_.resize(pat_.src.size());
    else d_vals_df_.release();
    launch_gather_values((int64_t)pat_.src.size(), d_src_.data(), d_csc_.data(), d_vals_.data(),
                         p_.mixed ? d_vals32_.data() : nullptr, stream_, df ? d_vals_df_.data() : nullptr);
    A_.vals = d_vals_.data();
    A_.vals32 = p_.mixed ? d_vals32_.data() : nullptr;
    A_.vals_df = df ? d_vals_df_.data() : nullptr;
    int bad = 0;
    LSS_CUDA(cudaMemcpyAsync(&bad, d_bad_.data(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    if (bad) fail(LSS_ERR_NONFINITE, "the matrix holds NaN or Inf values");
    auto t2 = clk::now();
    CscView A{pat_.n, pat_.nnz, h_outer_.data(), h_inner_.data(), nullptr};
    select_stiff(A);
    stats_["time_bad_dof_selection"] = secs(t2);
    auto t3 = clk::now();
    setup_stiff();
    LSS_CUDA(cudaStreamSynchronize(stream_));
    stats_["time_factorize_submatrix"] = secs(t3);
    auto t4 = clk::now();
    setup_mas();
    LSS_CUDA(cudaStreamSynchronize(stream_));
    stats_["time_mas_setup"] = secs(t4);
    setup_precise_rows();
    ensure_vectors();
    // d_csc_ stays allocated: the next factorization of this pattern (Newton
    // steps) reuses it instead of a cudaMalloc / cudaFree pair of nnz doubles
    factorized_ = true;
    if (!lanes_tuned_) autotune_spmv();
    auto t5 = clk::now();
    estimate_omega();
    stats_["time_omega_estimate"] = secs(t5);
    stats_["time_factorize_device"] = secs(t0);
}

void HybridSolver::set_problematic_dofs(const int32_t *idx, int32_t count)
{
    if (count < 0 || (count > 0 && !idx)) fail(LSS_ERR_INVALID_ARGUMENT, "invalid problematic DOF list");
    user_dofs_.assign(idx, idx + count);
    std::sort(user_dofs_.begin(), user_dofs_.end());
    user_dofs_.erase(std::unique(user_dofs_.begin(), user_dofs_.end()), user_dofs_.end());
}

void HybridSolver::select_stiff(const CscView &A)
{
    gmm_sel_.clear();
    subs_.clear();
    if (!p_.do_hybrid) return;
    if (p_.bad_dof_strategy != BADDOF_GPUHYBRID) {
        select_stiff_mas(A);
        return;
    }
    std::vector<int32_t> sel;
    auto tsel0 = clk::now();
    if (p_.select_l1) {
        const int32_t n = A.n;
        DBuf<double> rn(n);
        DBuf<GmmState> st(1);
        st.zero(stream_);
        if (d_outer_.size() != (size_t)n + 1) d_outer_.upload(h_outer_, stream_);
        launch_row_l1_norms(n, A.nnz, d_outer_.data(), d_csc_.data(), rn.data(), stream_);
        launch_gmm(n, rn.data(), st.data(), p_.max_gmm_iterations, p_.gmm_tol, gr_, stream_);
        const int nblk = (n + 255) / 256;
        DBuf<int32_t> bcount(nblk), boffs(nblk);
        DBuf<double> bmargin(nblk);
        launch_gmm_mark(n, rn.data(), st.data(), p_.jump_threshold, bcount.data(), bmargin.data(), stream_);
        std::vector<int32_t> hc = bcount.download(stream_);
        std::vector<double> hm = bmargin.download(stream_);
        std::vector<GmmState> hs = st.download(stream_);
        std::vector<int32_t> ho(nblk);
        int64_t total = 0;
        for (int b = 0; b < nblk; ++b) {
            ho[b] = (int32_t)total;
            total += hc[b];
        }
        double margin = INFINITY;
        for (double m : hm) margin = std::min(margin, m);
        sel.resize(total);
        if (total > 0) {
            boffs.upload(ho, stream_);
            DBuf<int32_t> out(total);
            launch_gmm_scatter(n, rn.data(), st.data(), p_.jump_threshold, boffs.data(), out.data(), stream_);
            sel = out.download(stream_);
        }
        const GmmState &g = hs[0];
        stats_["gmm_global_mean"] = g.mean;
        stats_["gmm_global_var"] = g.var;
        stats_["gmm_mean_0"] = g.m0;
        stats_["gmm_mean_1"] = g.m1;
        stats_["gmm_var_0"] = g.v0;
        stats_["gmm_var_1"] = g.v1;
        stats_["gmm_iters"] = g.converged ? g.esteps - 1 : g.esteps;
        stats_["gmm_min_log_margin"] = std::isfinite(margin) ? margin : -1.0;
    } else {
        for (int32_t v : user_dofs_)
            if (v >= 0 && v < A.n) sel.push_back(v);
    }
    gmm_sel_ = sel;
    stats_["time_selection_gmm"] = secs(tsel0);
    auto tsel1 = clk::now();
    // GPUHybrid.cu:221-238
    if (p_.decompose) {
        const int32_t m = (int32_t)sel.size();
        std::vector<double> diag(m), off(m);
        if (m > 0) {
            DBuf<int32_t> dsel;
            dsel.upload(sel, stream_);
            DBuf<uint8_t> mask((size_t)pat_.n);
            mask.zero(stream_);
            DBuf<double> ddiag(m), doff(m);
            launch_gershgorin(pat_.nb, pat_.bd, d_rows_.data(), d_cols_.data(), d_vals_.data(), d_perm_.data(),
                              dsel.data(), m, mask.data(), ddiag.data(), doff.data(), stream_);
            diag = ddiag.download(stream_);
            off = doff.download(stream_);
        }
        FilterCounters fc;
        sel = filter_subdomains(A, sel, diag, off, p_.min_sub, p_.max_sub, p_.cond_threshold, &fc);
        stats_["filter_too_small"] = fc.too_small;
        stats_["filter_too_large"] = fc.too_large;
        stats_["filter_not_poorly_conditioned"] = fc.not_poorly_conditioned;
    }
    stats_["time_selection_filter"] = secs(tsel1);
    auto tsel2 = clk::now();
    if (p_.expand && !sel.empty()) sel = expand_subdomains(A, sel);
    stats_["time_selection_expand"] = secs(tsel2);
    if (sel.empty()) return;
    // Without decompose_subdomains the reference factors one block with every
    // selected DOF; its inverse is block diagonal over the connected components,
    // so factoring the components separately applies the same operator.
    auto tsel3 = clk::now();
    // the components depend only on the pattern and the set: a factorization
    // that selects the same set as the previous one (same pattern) reuses them
    const int64_t max_size = p_.decompose ? (int64_t)p_.max_sub : INT64_MAX;
    if (sel == decomp_sel_ && max_size == decomp_max_) {
        subs_ = decomp_subs_;
    } else {
        subs_ = decompose_subdomains(A, sel, max_size);
        decomp_sel_ = sel;
        decomp_max_ = max_size;
        decomp_subs_ = subs_;
    }
    stats_["time_selection_decompose"] = secs(tsel3);
}

// MASSolver's bad-DOF selections (MASSolver.cu:266-290 with
// BadDOFPreconditioner / BadDofKMeanPreconditioner / BadDofGMMPreconditioner):
// scores per scalar row of the permuted operator on the device, selection on
// the host in that order (the expansion window counts partition-order
// positions), then one factorization of the selected set -- here its
// connected components, the same operator (components above
// bad_dof_max_block DOFs, beyond a dense inverse, are dropped).
void HybridSolver::select_stiff_mas(const CscView &A)
{
    const int64_t n = n_vec();
    const std::vector<double> score = row_scores(p_.bad_dof_strategy);
    std::vector<int32_t> pos;
    switch (p_.bad_dof_strategy) {
    case BADDOF_ELBOW: pos = mas_select_elbow(score); break;
    case BADDOF_KMEAN:
        pos = mas_select_kmean(score, p_.kmeans_search_fraction, p_.kmeans_jump_threshold, p_.kmeans_max_iterations,
                               p_.kmeans_expand_neighbors);
        break;
    default:
        pos = mas_select_gmm(score, p_.mas_gmm_jump_threshold, p_.mas_gmm_tol, p_.mas_gmm_max_iterations,
                             p_.mas_gmm_expand_neighbors);
        break;
    }
    const int32_t bd = pat_.bd;
    std::vector<int32_t> old_of(pat_.nb);
    for (int32_t b = 0; b < pat_.nb; ++b) old_of[pat_.part.perm[b]] = b;
    std::vector<int32_t> sel;
    sel.reserve(pos.size());
    for (int32_t p : pos)
        if (p >= 0 && p < n) sel.push_back(old_of[p / bd] * bd + p % bd);
    std::sort(sel.begin(), sel.end());
    gmm_sel_ = sel;
    stats_["bad_dof_selected"] = (double)sel.size();
    if (sel.empty()) return;
    subs_ = decompose_subdomains(A, sel, (int64_t)p_.bad_dof_max_block);
}

// kind 1: |diagonal|, 2: max |off-diagonal|, 3: l1 norm; per scalar row of the
// permuted operator
std::vector<double> HybridSolver::row_scores(int kind)
{
    const int64_t n = n_vec();
    DBuf<double> diag(n), offmax(n), l1(n);
    launch_row_scores(A_, diag.data(), offmax.data(), l1.data(), stream_);
    std::vector<double> out = (kind == BADDOF_ELBOW ? diag : (kind == BADDOF_KMEAN ? offmax : l1)).download(stream_);
    LSS_CUDA(cudaStreamSynchronize(stream_));
    return out;
}

void HybridSolver::op_row_scores(double *diag, double *offmax, double *l1)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "no factorized operator");
    const std::vector<double> a = row_scores(BADDOF_ELBOW), b = row_scores(BADDOF_KMEAN), c = row_scores(BADDOF_GMM);
    std::copy(a.begin(), a.end(), diag);
    std::copy(b.begin(), b.end(), offmax);
    std::copy(c.begin(), c.end(), l1);
}

void HybridSolver::setup_stiff()
{
    const int bd = pat_.bd;
    // the layout: subdomains with a dense inverse first, then those of the
    // multifrontal factor; DOFs permuted and ascending within each subdomain
    std::vector<int32_t> order;
    for (int pass = 0; pass < 2; ++pass)
        for (size_t s = 0; s < subs_.size(); ++s)
            if ((subs_[s].size() > (size_t)STIFF_DENSE_MAX) == (pass == 1)) order.push_back((int32_t)s);
    std::vector<int32_t> dofs, sub_of, off{0};
    std::vector<int64_t> inv_off;
    int64_t inv_total = 0;
    int32_t ndense = 0;
    for (size_t k = 0; k < order.size(); ++k) {
        const auto &sub = subs_[order[k]];
        std::vector<int32_t> d(sub.size());
        for (size_t q = 0; q < d.size(); ++q) {
            const int32_t g = sub[q];
            d[q] = pat_.part.perm[g / bd] * bd + g % bd;
        }
        std::sort(d.begin(), d.end());
        const bool dense = d.size() <= (size_t)STIFF_DENSE_MAX;
        dofs.insert(dofs.end(), d.begin(), d.end());
        sub_of.insert(sub_of.end(), d.size(), (int32_t)k);
        off.push_back((int32_t)dofs.size());
        inv_off.push_back(inv_total);
        if (dense) {
            inv_total += (int64_t)d.size() * (int64_t)d.size();
            ++ndense;
        }
    }
    // the same stiff subdomains as the previous factorization (repeated
    // factorizations of one pattern, e.g. Newton steps): the device layout,
    // the multifrontal plan and its storage are kept, only the numbers change
    const bool same = !subs_.empty() && mf_ && dofs == h_sdofs_ && off == h_soff_ && ndense == ndense_;
    if (!same) {
        stiff_ = StiffDev();
        d_sdofs_.release();
        d_ssub_.release();
        d_soff_.release();
        d_sinvoff_.release();
        d_sinv_.release();
        d_sinv32_.release();
        d_st_.release();
        mf_ = std::make_unique<MfFactor>();
        h_sdofs_.clear();
        h_soff_.assign(1, 0);
        h_sinvoff_.clear();
        ndense_ = 0;
        inv_total_ = 0;
        if (subs_.empty()) return;
        d_sdofs_.upload(dofs, stream_);
        d_ssub_.upload(sub_of, stream_);
        d_soff_.upload(off, stream_);
        d_sinvoff_.upload(inv_off, stream_);
        d_sinv_.resize(std::max<int64_t>(inv_total, 1));
        d_st_.resize(dofs.size());
        stiff_.nsub = (int32_t)order.size();
        stiff_.ndof = (int32_t)dofs.size();
        stiff_.ndof_dense = off[ndense];
        stiff_.dofs = d_sdofs_.data();
        stiff_.sub_of = d_ssub_.data();
        stiff_.off = d_soff_.data();
        stiff_.inv_off = d_sinvoff_.data();
        stiff_.inv = d_sinv_.data();
        stiff_.t = d_st_.data();
    }
    stats_["stiff_layout_reused"] = same ? 1.0 : 0.0;
    d_sinv_.zero(stream_);
    d_bad_.zero(stream_);
    launch_stiff_extract(A_, stiff_, d_sinv_.data(), stream_);
    launch_stiff_invert(stiff_, off.data(), ndense, d_sinv_.data(), d_bad_.data(), stream_);
    if (ndense < stiff_.nsub) {
        if (!same) {
            auto t0 = clk::now();
            const MfSymbolic sym = mf_symbolic(dofs, off, ndense, pat_.rows, pat_.cols, bd);
            stats_["time_multifrontal_symbolic"] = secs(t0);
            mf_->setup(sym, stream_);
        } else {
            stats_["time_multifrontal_symbolic"] = 0.0;
        }
        mf_->factorize(A_, stiff_, d_bad_.data(), stream_);
        const MfSymbolic &sym = mf_->symbolic();
        stats_["multifrontal_fronts"] = sym.nfront;
        stats_["multifrontal_levels"] = sym.levels;
        stats_["multifrontal_max_front"] = sym.max_f;
        stats_["multifrontal_fmas"] = sym.fmas;
        stats_["multifrontal_bytes"] = (double)mf_->bytes();
    }
    int bad = 0;
    LSS_CUDA(cudaMemcpyAsync(&bad, d_bad_.data(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    if (bad) fail(LSS_ERR_NOT_SPD, "a stiff subdomain block has a zero or non-finite pivot");
    if (p_.float_subdomains && inv_total > 0) {
        d_sinv32_.resize(inv_total);
        launch_stiff_to_fp32(inv_total, d_sinv_.data(), d_sinv32_.data(), stream_);
        stiff_.inv32 = d_sinv32_.data();
    }
    int64_t maxm = 0;
    for (const auto &sub : subs_) maxm = std::max<int64_t>(maxm, (int64_t)sub.size());
    stats_["max_subdomain_dofs"] = (double)maxm;
    stats_["dense_subdomains"] = ndense;
    h_sdofs_ = std::move(dofs);
    h_soff_ = std::move(off);
    h_sinvoff_ = std::move(inv_off);
    ndense_ = ndense;
    inv_total_ = inv_total;
    stats_["multifrontal_subdomains"] = stiff_.nsub - ndense;
}

// z_S += A_SS^-1 t over every stiff subdomain (dense inverses and the
// multifrontal factor; disjoint DOF sets)
void HybridSolver::stiff_correct(double *z, const int *done, float *z32, float *z_lo)
{
    launch_stiff_apply(stiff_, p_.float_subdomains, z, done, stream_, z32, z_lo);
    if (mf_ && !mf_->empty()) mf_->solve(stiff_, z, z32, z_lo, done, stream_);
}

// Mixed precision: the block rows whose preconditioner residual runs in
// double-float -- every block row holding a DOF of the GMM selection or of a
// stiff subdomain ("auto"), all rows ("df32") or none ("fp32").
void HybridSolver::setup_precise_rows()
{
    precise_rows_ = false;
    h_precise_.clear();
    if (!p_.mixed || p_.precond_residual == 1) {
        d_precise_.release();
        return;
    }
    const int32_t nb = pat_.nb, bd = pat_.bd;
    std::vector<uint8_t> flag(nb, p_.precond_residual == 2 ? 1 : 0);
    int64_t count = p_.precond_residual == 2 ? nb : 0;
    auto mark = [&](int32_t dof) {
        if (dof < 0 || dof >= pat_.n) return;
        uint8_t &f = flag[pat_.part.perm[dof / bd]];
        if (!f) {
            f = 1;
            ++count;
        }
    };
    if (p_.precond_residual == 0) {
        for (int32_t d : gmm_sel_) mark(d);
        for (const auto &s : subs_)
            for (int32_t d : s) mark(d);
    }
    stats_["precise_residual_block_rows"] = (double)count;
    h_precise_ = flag;
    if (count == 0) {
        d_precise_.release();
        return;
    }
    d_precise_.upload(flag, stream_);
    precise_rows_ = true;
}

void HybridSolver::setup_mas()
{
    const int bd = pat_.bd, N = 32 * bd;
    const int64_t nparts = mas_.nparts, ncoarse = mas_.ncoarse;
    const int64_t te = mas_.tile_elems;
    const size_t esz = mas_fp32_ ? sizeof(float) : sizeof(double);
    // mixed precision may store the level-0 off-diagonal tiles in BF16
    const bool bf = mas_fp32_ && p_.mas_bf16_offdiag && bd > 1;
    mas_.bank_bytes0 = bf ? mas_bank_bytes_bf16(bd) : 0;
    d_inv0_.resize(bf ? (size_t)(nparts * mas_.bank_bytes0) : (size_t)(nparts * te * esz));
    d_invc_.resize(std::max<int64_t>(ncoarse, 1) * te * esz);
    d_bad_.zero(stream_);
    // the dense staging of the Galerkin blocks stays allocated across the
    // factorizations of a pattern (no cudaMalloc / cudaFree of GBs per step)
    {
        // level 0 (no atomics: every entry comes from its own row)
        d_stage0_.resize((size_t)nparts * N * N);
        d_stage0_.zero(stream_);
        launch_mas_assemble0(A_, d_part_of_.data(), d_part_off_.data(), d_stage0_.data(), stream_);
        launch_mas_invert(bd, nparts, d_stage0_.data(), d_inv0_.data(), mas_fp32_, d_bad_.data(), stream_, bf);
    }
    if (ncoarse > 0) {
        d_stagec_.resize((size_t)ncoarse * N * N);
        d_stagec_.zero(stream_);
        d_cpartial_.resize((size_t)std::max<int64_t>(memb_.nchunk, 1) * bd * bd * 32);
        launch_mas_assemble_coarse(A_, mas_, d_cmap_.data(), memb_, d_cpartial_.data(), d_stagec_.data(), stream_);
        launch_mas_invert(bd, ncoarse, d_stagec_.data(), d_invc_.data(), mas_fp32_, d_bad_.data(), stream_);
    }
    int bad = 0;
    LSS_CUDA(cudaMemcpyAsync(&bad, d_bad_.data(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    if (bad) fail(LSS_ERR_NOT_SPD, "[MAS] packed inverse failed (zero or non-finite pivot)");
    d_v_.resize(std::max<int64_t>(mas_.level_elems, 1) * esz);
    d_u_.resize(std::max<int64_t>(mas_.level_elems, 1) * esz);
    d_v_.zero(stream_);
    d_u_.zero(stream_);
    stats_["mas_inverse_bytes"] = (double)(bf ? nparts * mas_.bank_bytes0 : nparts * te * esz) + (double)ncoarse * te * esz;
}

void HybridSolver::ensure_vectors()
{
    const int64_t n = n_vec();
    for (DBuf<double> *b : {&d_x_, &d_b_, &d_r_, &d_p_, &d_z_, &d_ap_, &d_w_, &d_tmp_}) b->resize(n);
    for (DBuf<float> *b : {&d_z32_, &d_r32_, &d_w32_, &d_z_lo_}) {
        if (p_.mixed) {
            b->resize(n);
            b->zero(stream_);
        } else {
            b->release();
        }
    }
    for (DBuf<float2> *b : {&d_p_df_, &d_ap_df_}) {
        if (df32()) b->resize(n);
        else b->release();
    }
}

// ------------------------------------------------------------------ preconditioner

void HybridSolver::mas_apply(const double *xin, double *z, bool acc, const double *rdot, int dot_mode, double scale,
                             float *z32, const float *xin32, float *z_lo)
{
    launch_mas_apply(mas_, d_inv0_.data(), d_invc_.data(), d_v_.data(), d_u_.data(), mas_fp32_, xin, z, acc, scale,
                     rdot, d_state_.data(), dot_mode, gr_, &d_state_.data()->done, stream_, z32, xin32, z_lo);
}

void HybridSolver::rz_dot(const double *r, const double *z, int dot_mode)
{
    launch_pcg_rz(n_vec(), r, z, d_state_.data(), dot_mode, gr_, stream_);
}

// z = M^-1 r.  dot_mode 0: nothing; 1: gamma = r.z; 2: beta, gamma update.
void HybridSolver::precond(const double *r, double *z, int dot_mode, const float *r32)
{
    const int *done = &d_state_.data()->done;
    const bool stiff = p_.do_hybrid && stiff_.ndof > 0 && !lanczos_mode_;
    if (!stiff) {  // GPUHybrid.cu:523-527
        mas_apply(r, z, false, r, dot_mode, 1.0);
        return;
    }
    if (!p_.multiplicative) {  // MASSolver.cu:583-615: z = M r + S^T A_SS^-1 S r
        mas_apply(r, z, false, nullptr, 0, 1.0);
        launch_stiff_gather(A_, stiff_, r, nullptr, false, done, stream_);
        stiff_correct(z, done);
        if (dot_mode) rz_dot(r, z, dot_mode);
        return;
    }
    // GPUHybrid.cu:528-540 with omega-damped MAS in place of the V-cycle:
    // z1 = w M r; z2 = z1 + S^T A_SS^-1 S (r - A z1); z = z2 + w M (r - A z2).
    // The symmetric product is SPD when I - w M A contracts in the A-norm;
    // additive MAS has lambda_max(M A) of a few units, so w = omega_factor /
    // lambda_max(M A) is estimated at factorize time (estimate_omega).
    if (!p_.mixed) {
        mas_apply(r, z, false, nullptr, 0, omega_);
        launch_stiff_gather(A_, stiff_, r, z, true, done, stream_);
        stiff_correct(z, done);
        launch_residual_spmv(A_, r, z, d_w_.data(), done, stream_);
        mas_apply(d_w_.data(), z, true, r, dot_mode, omega_);
        return;
    }
    // mixed precision: z also goes out rounded to FP32 (the stiff correction
    // keeps that copy current) and r - A z runs entirely in FP32 into the
    // second, FP32 MAS apply; no FP64 instruction is spent on conversions
    // inside the SpMV (r32 comes from the PCG update, or is converted here).
    if (!r32) {
        launch_stiff_to_fp32(n_vec(), r, d_r32_.data(), stream_);
        r32 = d_r32_.data();
    }
    float *z32 = d_z32_.data();
    float *z_lo = precise_rows_ ? d_z_lo_.data() : nullptr;
    mas_apply(r, z, false, nullptr, 0, omega_, z32, nullptr, z_lo);
    launch_stiff_gather(A_, stiff_, r, z, true, done, stream_);
    stiff_correct(z, done, z32, z_lo);
    launch_residual32(A_, r32, z32, d_w32_.data(), done, stream_, precise_rows_ ? d_precise_.data() : nullptr, r,
                      z_lo);
    mas_apply(nullptr, z, true, r, dot_mode, omega_, nullptr, d_w32_.data());
}

// ------------------------------------------------------------------ PCG

void HybridSolver::outer_spmv_alpha()
{
    if (outer_df())
        launch_pcg_spmv_alpha_df(A_, d_p_df_.data(), d_ap_df_.data(), d_state_.data(), gr_, stream_);
    else
        launch_pcg_spmv_alpha(A_, d_p_.data(), d_ap_.data(), d_state_.data(), gr_, stream_);
}

void HybridSolver::split_p()
{
    if (outer_df()) launch_split(n_vec(), d_p_.data(), d_p_df_.data(), stream_);
}

void HybridSolver::iteration()
{
    outer_spmv_alpha();
    float *r32 = p_.mixed ? d_r32_.data() : nullptr;
    if (outer_df())
        launch_pcg_update_xr_df(n_vec(), d_x_.data(), d_r_.data(), d_p_.data(), d_ap_df_.data(), d_state_.data(),
                                gr_, stream_, r32);
    else
        launch_pcg_update_xr(n_vec(), d_x_.data(), d_r_.data(), d_p_.data(), d_ap_.data(), d_state_.data(), gr_,
                             stream_, r32);
    precond(d_r_.data(), d_z_.data(), 2, r32);
    launch_pcg_update_p(n_vec(), d_p_.data(), d_z_.data(), d_state_.data(), stream_,
                        outer_df() ? d_p_df_.data() : nullptr);
}

void HybridSolver::launch_chunk(int iters)
{
    if (!p_.use_graphs) {
        for (int k = 0; k < iters; ++k) iteration();
        return;
    }
    if (!graph_exec_ || graph_iters_ != iters) {
        invalidate_graph();
        cudaGraph_t g = nullptr;
        LSS_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        try {
            for (int k = 0; k < iters; ++k) iteration();
        } catch (...) {
            cudaStreamEndCapture(stream_, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        LSS_CUDA(cudaStreamEndCapture(stream_, &g));
        size_t nodes = 0;
        if (cudaGraphGetNodes(g, nullptr, &nodes) == cudaSuccess) stats_["kernels_per_iteration"] = (double)nodes / iters;
        graph_nodes_ = nodes;
        // the capture ran the launchers once without executing anything
        launch_count() -= std::min<unsigned long long>(launch_count().load(), nodes);
        LSS_CUDA(cudaGraphInstantiate(&graph_exec_, g, 0));
        cudaGraphDestroy(g);
        graph_iters_ = iters;
    }
    LSS_CUDA(cudaGraphLaunch(graph_exec_, stream_));
    launch_count() += graph_nodes_;
}

void HybridSolver::run_pcg()
{
    // the refinement restarts switch the outer product to FP64; every solve
    // starts with the configured one
    struct RefineReset {
        HybridSolver *s;
        ~RefineReset()
        {
            if (s->refine_fp64_) {
                s->refine_fp64_ = false;
                s->invalidate_graph();
            }
        }
    } refine_reset{this};
    const int64_t n = n_vec();
    double *bb_d = d_scalar_.data();
    launch_dot(n, d_b_.data(), d_b_.data(), bb_d, gr_, stream_);
    double bb = 0.0;
    LSS_CUDA(cudaMemcpyAsync(&bb, bb_d, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    if (!std::isfinite(bb)) fail(LSS_ERR_NONFINITE, "the right-hand side holds NaN or Inf values");
    rhs_norm_ = std::sqrt(bb);
    refinements_ = 0;
    if (!(bb > 0.0)) {  // GPUHybrid.cu:1428-1439
        d_x_.zero(stream_);
        num_iterations_ = 0;
        final_res_norm_ = 0.0;
        stop_reason_ = STOP_CONVERGED_ABS;
        LSS_CUDA(cudaStreamSynchronize(stream_));
        return;
    }
    PcgState hs{};
    hs.bb = bb;
    hs.rel_eps = p_.rel_tol * p_.rel_tol;
    hs.abs_eps = p_.abs_tol * p_.abs_tol;
    hs.max_iter = p_.max_iter;
    hs.iter = 0;
    hs.done = STOP_RUNNING;
    *h_state_ = hs;
    LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    int launched = 0;
    double res2 = 0.0, prev_res2 = INFINITY;
    for (int attempt = 0;; ++attempt) {
        // r = b - A x; z = M r; p = z; gamma = r.z   (GPUHybrid.cu:1441-1451)
        launch_residual_spmv(A_, d_b_.data(), d_x_.data(), d_r_.data(), nullptr, stream_);
        if (p_.max_iter > 0) {
            precond(d_r_.data(), d_z_.data(), 1);
            launch_copy(n, d_z_.data(), d_p_.data(), nullptr, stream_);
            split_p();
        }
        while (launched < p_.max_iter) {
            const int chunk = std::min(p_.check_every, p_.max_iter - launched);
            launch_chunk(chunk);
            launched += chunk;
            LSS_CUDA(cudaMemcpyAsync(h_state_, d_state_.data(), sizeof(PcgState), cudaMemcpyDeviceToHost, stream_));
            LSS_CUDA(cudaStreamSynchronize(stream_));
            if (h_state_->done) break;
        }
        // true residual (GPUHybrid.cu:383-386)
        launch_residual_spmv(A_, d_b_.data(), d_x_.data(), d_w_.data(), nullptr, stream_);
        launch_dot(n, d_w_.data(), d_w_.data(), bb_d, gr_, stream_);
        LSS_CUDA(cudaMemcpyAsync(&res2, bb_d, sizeof(double), cudaMemcpyDeviceToHost, stream_));
        LSS_CUDA(cudaMemcpyAsync(h_state_, d_state_.data(), sizeof(PcgState), cudaMemcpyDeviceToHost, stream_));
        LSS_CUDA(cudaStreamSynchronize(stream_));
        const int reason = h_state_->done;
        const bool converged = reason == STOP_CONVERGED_REL || reason == STOP_CONVERGED_ABS;
        // 2% margin: a second FP64 evaluation of b - A x (another summation
        // order) must not find the returned x above the tolerance
        const bool true_ok = !(hs.rel_eps > 0) || res2 / bb <= 0.9604 * hs.rel_eps;
        // restart only while restarting still pays: the true residual has a rounding
        // floor of about eps * || |A| |x| || that no restart can go below
        const bool improving = res2 < 0.25 * prev_res2;
        prev_res2 = res2;
        if (converged && !true_ok && improving && attempt < p_.max_refinements && launched < p_.max_iter) {
            // the recurrence residual drifted from the true one: restart from x,
            // aiming the recurrence below the tolerance by the drift seen so far
            // (at least 2x), so that the restarted solve's own drift still lands
            // the true residual under it
            ++refinements_;
            h_state_->done = STOP_RUNNING;
            // the restarts use the FP64 product: the double-float one's 2^-48 per
            // term sets a floor of 2^-48 || |A| |x| || that can exceed the
            // tolerance on high-contrast systems (1e7 moduli times a near-rigid x)
            if (outer_df()) {
                refine_fp64_ = true;
                invalidate_graph();
            }
            if (hs.rel_eps > 0 && !true_ok) {
                const double true_rel = std::sqrt(res2 / bb);
                const double target = p_.rel_tol * std::min(1.0, 0.5 * p_.rel_tol / true_rel);
                h_state_->rel_eps = target * target;
            }
            LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
            continue;
        }
        break;
    }
    num_iterations_ = h_state_->iter;
    stop_reason_ = h_state_->done ? h_state_->done : STOP_MAX_ITER;
    final_res_norm_ = std::sqrt(res2);
}

// Autotuner of the SpMV launch shape: threads per block row in {1, 2, 4, 8, 16}
// for the FP64 operator and the FP32 copy, timed with CUDA events on the real
// matrix once per pattern.  Fewer lanes mean more blocks per lane (more
// independent loads in flight) and a shallower cross-lane FP64 reduction --
// which matters on a GPU whose FP64 rate is 1/57 of its FP32 rate.
namespace {
// Tuned launch shapes per (pattern, block size, operator form), shared by the
// solvers of a process: the lanes decide the summation order of every row, so
// reusing the first choice keeps a second solver of the same system
// bit-identical to the first (timings alone could pick differently).
struct TuneKey {
    uint64_t hash;
    int64_t nnz;
    int bd, mixed, df, device;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(hash, nnz, bd, mixed, df, device) < std::tie(o.hash, o.nnz, o.bd, o.mixed, o.df, o.device);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, int>> g_tuned;
}  // namespace

void HybridSolver::autotune_spmv()
{
    const TuneKey key{pat_.hash, pat_.nnz, pat_.bd, p_.mixed ? 1 : 0, df32() ? 1 : 0, p_.device};
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            A_.lanes = it->second.first;
            A_.lanes32 = it->second.second;
            lanes_tuned_ = true;
            sstats_["spmv_autotune_ms"] = "cached";
            return;
        }
    }
    const int64_t n = n_vec();
    std::vector<double> h(n);
    for (int64_t i = 0; i < n; ++i) h[i] = 1.0 + 1e-3 * (double)(i % 89);
    LSS_CUDA(cudaMemcpyAsync(d_p_.data(), h.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_r_.data(), h.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    if (p_.mixed) {
        launch_stiff_to_fp32(n, d_p_.data(), d_z32_.data(), stream_);
        launch_stiff_to_fp32(n, d_r_.data(), d_r32_.data(), stream_);
    }
    cudaEvent_t e0, e1;
    LSS_CUDA(cudaEventCreate(&e0));
    LSS_CUDA(cudaEventCreate(&e1));
    auto time_it = [&](auto &&launch) {
        launch();
        LSS_CUDA(cudaEventRecord(e0, stream_));
        for (int k = 0; k < 5; ++k) launch();
        LSS_CUDA(cudaEventRecord(e1, stream_));
        LSS_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        LSS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return ms;
    };
    std::string log;
    if (df32()) {
        split_p();
        PcgState hs{};
        hs.gamma = 1.0;
        hs.max_iter = 1 << 30;
        *h_state_ = hs;
        LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    }
    for (int pass = 0; pass < (p_.mixed ? 2 : 1); ++pass) {
        float best = 1e30f;
        int best_l = 4;
        for (int l : {1, 2, 4, 8, 16}) {
            BsrDev T = A_;
            T.lanes = T.lanes32 = l;
            const float ms = pass == 0 ? time_it([&]() {
                                             if (df32())
                                                 launch_pcg_spmv_alpha_df(T, d_p_df_.data(), d_ap_df_.data(),
                                                                          d_state_.data(), gr_, stream_);
                                             else
                                                 launch_spmv(T, d_p_.data(), d_ap_.data(), nullptr, stream_);
                                         })
                                       : time_it([&]() {
                                             launch_residual32(T, d_r32_.data(), d_z32_.data(), d_w32_.data(),
                                                               nullptr, stream_,
                                                               precise_rows_ ? d_precise_.data() : nullptr,
                                                               d_r_.data(), d_z_lo_.data());
                                         });
            log += (pass ? " f32:" : (df32() ? " df32:" : " f64:")) + std::to_string(l) + "=" + std::to_string(ms / 5);
            if (ms < best) { best = ms; best_l = l; }
        }
        if (pass == 0) A_.lanes = best_l;
        else A_.lanes32 = best_l;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    lanes_tuned_ = true;
    sstats_["spmv_autotune_ms"] = log;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned.emplace(key, std::make_pair(A_.lanes, A_.lanes32));
}

// lambda_max(M A) for M = MAS alone from the Lanczos tridiagonal of a short
// PCG run on a fixed probe vector (CG coefficients a_j, b_j give diagonal
// 1/a_j + b_{j-1}/a_{j-1} and off-diagonal sqrt(b_j)/a_j); largest eigenvalue
// of the tridiagonal by bisection on Sturm counts.
static double tridiag_max_eig(int k, const double *d, const double *e)
{
    if (k <= 0) return 0.0;
    double lo = d[0], hi = d[0];
    for (int j = 0; j < k; ++j) {
        const double r = (j > 0 ? std::fabs(e[j - 1]) : 0.0) + (j + 1 < k ? std::fabs(e[j]) : 0.0);
        lo = std::min(lo, d[j] - r);
        hi = std::max(hi, d[j] + r);
    }
    auto count_below = [&](double x) {
        int c = 0;
        double q = d[0] - x;
        if (q < 0) ++c;
        for (int j = 1; j < k; ++j) {
            if (q == 0.0) q = 1e-300;
            q = d[j] - x - e[j - 1] * e[j - 1] / q;
            if (q < 0) ++c;
        }
        return c;
    };
    for (int it = 0; it < 200 && hi - lo > 1e-14 * std::fabs(hi); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (count_below(mid) >= k) hi = mid;
        else lo = mid;
    }
    return hi;
}

void HybridSolver::estimate_omega()
{
    omega_ = 1.0;
    lambda_max_ = 0.0;
    if (!(p_.do_hybrid && stiff_.ndof > 0 && p_.multiplicative)) return;
    if (p_.mas_damping > 0) {
        omega_ = p_.mas_damping;
        return;
    }
    const int64_t n = n_vec();
    const int k = p_.omega_iters;
    // probe vector v_i = ((i * 2654435761) mod 2^32) / 2^32 - 0.5, original ordering
    launch_probe(pat_.nb, pat_.bd, d_perm_.data(), d_r_.data(), stream_);
    PcgState hs{};
    hs.bb = 1.0;
    hs.max_iter = k;
    *h_state_ = hs;
    LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    d_x_.zero(stream_);
    lanczos_mode_ = true;
    try {
        precond(d_r_.data(), d_z_.data(), 1);
        launch_copy(n, d_z_.data(), d_p_.data(), nullptr, stream_);
        split_p();
        for (int j = 0; j < k; ++j) iteration();
    } catch (...) {
        lanczos_mode_ = false;
        throw;
    }
    lanczos_mode_ = false;
    LSS_CUDA(cudaMemcpyAsync(h_state_, d_state_.data(), sizeof(PcgState), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    // usable steps: those with both coefficients recorded
    int m = std::min(h_state_->iter, k);
    std::vector<double> a(h_state_->hist_alpha, h_state_->hist_alpha + m);
    std::vector<double> b(h_state_->hist_beta, h_state_->hist_beta + m);
    int good = 0;
    while (good < m && a[good] > 0 && std::isfinite(a[good]) && std::isfinite(b[good]) && b[good] >= 0) ++good;
    std::vector<double> d(good), e(good > 0 ? good : 1);
    for (int j = 0; j < good; ++j) {
        d[j] = 1.0 / a[j] + (j > 0 ? b[j - 1] / a[j - 1] : 0.0);
        if (j + 1 < good) e[j] = std::sqrt(b[j]) / a[j];
    }
    lambda_max_ = tridiag_max_eig(good, d.data(), e.data());
    if (lambda_max_ > 0) omega_ = p_.omega_factor / lambda_max_;
    stats_["mas_lambda_max"] = lambda_max_;
    std::string hist;
    for (int j = 0; j < m; ++j) hist += (j ? " " : "") + std::to_string(a[j]) + "/" + std::to_string(b[j]);
    sstats_["omega_lanczos_alpha_beta"] = hist;
}

void HybridSolver::solve_host(const double *b, double *x)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "solve called before factorize");
    if (!b || !x) fail(LSS_ERR_INVALID_ARGUMENT, "null vector");
    auto t0 = clk::now();
    const int64_t n = n_vec();
    double *pin = (double *)pin_.get((size_t)n * sizeof(double) * 2);
    const int ht = host_threads();
    parallel_copy(pin, b, (size_t)n * sizeof(double), ht);
    parallel_copy(pin + n, x, (size_t)n * sizeof(double), ht);
    LSS_CUDA(cudaMemcpyAsync(d_tmp_.data(), pin, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_tmp_.data(), d_b_.data(), true, stream_);
    LSS_CUDA(cudaMemcpyAsync(d_tmp_.data(), pin + n, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_tmp_.data(), d_x_.data(), true, stream_);
    run_pcg();
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_x_.data(), d_tmp_.data(), false, stream_);
    LSS_CUDA(cudaMemcpyAsync(pin, d_tmp_.data(), (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    parallel_copy(x, pin, (size_t)n * sizeof(double), ht);
    stats_["time_solve"] = secs(t0);
}

void HybridSolver::solve_device(const double *d_b, double *d_x, cudaStream_t user)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "solve called before factorize");
    auto t0 = clk::now();
    StreamScope scope(this, user);
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_b, d_b_.data(), true, stream_);
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_x, d_x_.data(), true, stream_);
    run_pcg();
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_x_.data(), d_x, false, stream_);
    LSS_CUDA(cudaStreamSynchronize(stream_));
    stats_["time_solve"] = secs(t0);
}

void HybridSolver::grad_pattern_device(const double *d_lambda, const double *d_x, double *d_dA, cudaStream_t user)
{
    if (!have_pattern_) fail(LSS_ERR_NOT_FACTORIZED, "no matrix pattern");
    StreamScope scope(this, user);
    if (d_outer_.size() != h_outer_.size()) d_outer_.upload(h_outer_, stream_);
    if (d_inner_.size() != h_inner_.size()) d_inner_.upload(h_inner_, stream_);
    launch_grad_pattern(pat_.n, d_outer_.data(), d_inner_.data(), d_lambda, d_x, d_dA, stream_);
    LSS_CUDA(cudaStreamSynchronize(stream_));
}

void HybridSolver::grad_params_device(const double *d_lambda, const double *d_x, int32_t nparams,
                                      const int64_t *d_rowptr, const int32_t *d_cols, const double *d_vals,
                                      double *d_dtheta, cudaStream_t user)
{
    if (!have_pattern_) fail(LSS_ERR_NOT_FACTORIZED, "no matrix pattern");
    if (nparams < 0 || (nparams > 0 && (!d_rowptr || !d_cols || !d_vals || !d_dtheta)))
        fail(LSS_ERR_INVALID_ARGUMENT, "invalid parameter map");
    StreamScope scope(this, user);
    if (d_outer_.size() != h_outer_.size()) d_outer_.upload(h_outer_, stream_);
    if (d_inner_.size() != h_inner_.size()) d_inner_.upload(h_inner_, stream_);
    if (d_row_of_.size() != (size_t)pat_.nnz) {
        d_row_of_.resize(pat_.nnz);
        launch_row_of(pat_.n, d_outer_.data(), d_row_of_.data(), stream_);
    }
    launch_grad_params(nparams, d_rowptr, d_cols, d_vals, d_row_of_.data(), d_inner_.data(), d_lambda, d_x, d_dtheta,
                       stream_);
    LSS_CUDA(cudaStreamSynchronize(stream_));
}

void HybridSolver::grad_pattern_host(const double *lambda, const double *x, double *dA)
{
    if (!have_pattern_) fail(LSS_ERR_NOT_FACTORIZED, "no matrix pattern");
    // dL/dA_ij = -lambda_i x_j on the stored pattern (outer index = row)
    for (int32_t i = 0; i < pat_.n; ++i)
        for (int32_t k = h_outer_[i]; k < h_outer_[i + 1]; ++k) dA[k] = -lambda[i] * x[h_inner_[k]];
}

// ------------------------------------------------------------------ operator access

void HybridSolver::op_spmv(const double *x, double *y)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "no factorized operator");
    const int64_t n = n_vec();
    LSS_CUDA(cudaMemcpyAsync(d_tmp_.data(), x, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_tmp_.data(), d_p_.data(), true, stream_);
    launch_spmv(A_, d_p_.data(), d_ap_.data(), nullptr, stream_);
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_ap_.data(), d_tmp_.data(), false, stream_);
    LSS_CUDA(cudaMemcpyAsync(y, d_tmp_.data(), n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
}

void HybridSolver::op_spmv_outer(const double *x, double *y)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "no factorized operator");
    const int64_t n = n_vec();
    PcgState hs{};
    hs.gamma = 1.0;
    hs.max_iter = 1 << 30;
    *h_state_ = hs;
    LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_tmp_.data(), x, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_tmp_.data(), d_p_.data(), true, stream_);
    split_p();
    outer_spmv_alpha();
    if (outer_df()) launch_df_to_double(n, d_ap_df_.data(), d_ap_.data(), stream_);
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_ap_.data(), d_tmp_.data(), false, stream_);
    LSS_CUDA(cudaMemcpyAsync(y, d_tmp_.data(), n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
}

void HybridSolver::op_mas(const double *r, double *z)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "no factorized operator");
    const int64_t n = n_vec();
    PcgState hs{};
    *h_state_ = hs;
    LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_tmp_.data(), r, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_tmp_.data(), d_r_.data(), true, stream_);
    mas_apply(d_r_.data(), d_z_.data(), false, nullptr, 0, 1.0);
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_z_.data(), d_tmp_.data(), false, stream_);
    LSS_CUDA(cudaMemcpyAsync(z, d_tmp_.data(), n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
}

void HybridSolver::op_precond(const double *r, double *z)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "no factorized operator");
    const int64_t n = n_vec();
    PcgState hs{};
    *h_state_ = hs;
    LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_tmp_.data(), r, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_tmp_.data(), d_r_.data(), true, stream_);
    precond(d_r_.data(), d_z_.data(), 0);
    launch_permute(pat_.nb, pat_.bd, d_perm_.data(), d_z_.data(), d_tmp_.data(), false, stream_);
    LSS_CUDA(cudaMemcpyAsync(z, d_tmp_.data(), n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
}

void HybridSolver::op_time(int kind, int reps, double *ms, double *bytes)
{
    if (!factorized_) fail(LSS_ERR_NOT_FACTORIZED, "no factorized operator");
    if (reps < 1) reps = 1;
    const int64_t n = n_vec();
    const int bd = pat_.bd;
    const int64_t nnzb = pat_.rows.back();
    PcgState hs{};
    hs.bb = 1.0;
    hs.max_iter = 1 << 30;
    hs.gamma = 1.0;
    *h_state_ = hs;
    LSS_CUDA(cudaMemcpyAsync(d_state_.data(), h_state_, sizeof(PcgState), cudaMemcpyHostToDevice, stream_));
    // deterministic non-trivial operands
    std::vector<double> h(n);
    for (int64_t i = 0; i < n; ++i) h[i] = 1.0 + 1e-3 * (double)(i % 97);
    LSS_CUDA(cudaMemcpyAsync(d_p_.data(), h.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_r_.data(), h.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_x_.data(), h.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(d_z_.data(), h.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    if (p_.mixed) {
        launch_stiff_to_fp32(n, d_p_.data(), d_z32_.data(), stream_);
        launch_stiff_to_fp32(n, d_r_.data(), d_r32_.data(), stream_);
    }
    split_p();
    auto body = [&]() {
        switch (kind) {
        case 0: launch_spmv(A_, d_p_.data(), d_ap_.data(), nullptr, stream_); break;
        case 1: mas_apply(d_r_.data(), d_z_.data(), false, nullptr, 0, 1.0); break;
        case 2: precond(d_r_.data(), d_z_.data(), 0); break;
        case 4: launch_mas_level0(mas_, d_inv0_.data(), d_u_.data(), mas_fp32_, d_r_.data(), d_z_.data(), stream_);
            break;
        case 5:
            if (p_.mixed)
                launch_residual32(A_, d_r32_.data(), d_z32_.data(), d_w32_.data(), nullptr, stream_,
                                  precise_rows_ ? d_precise_.data() : nullptr, d_r_.data(), d_z_lo_.data());
            else launch_residual_spmv(A_, d_r_.data(), d_p_.data(), d_ap_.data(), nullptr, stream_);
            break;
        case 6: outer_spmv_alpha(); break;
        default: iteration(); break;
        }
    };
    body();
    cudaEvent_t e0, e1;
    LSS_CUDA(cudaEventCreate(&e0));
    LSS_CUDA(cudaEventCreate(&e1));
    LSS_CUDA(cudaEventRecord(e0, stream_));
    for (int k = 0; k < reps; ++k) body();
    LSS_CUDA(cudaEventRecord(e1, stream_));
    LSS_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    LSS_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / reps;
    const double spmv_bytes = (double)nnzb * (bd * bd * 8 + 4) + (pat_.nb + 1) * 4.0 + 2.0 * n * 8;
    const double esz = mas_fp32_ ? 4.0 : 8.0;
    const double inv0_bytes = mas_.bank_bytes0 > 0 ? (double)mas_.nparts * mas_.bank_bytes0
                                                   : (double)mas_.nparts * mas_.tile_elems * esz;
    const double mas_bytes = inv0_bytes + (double)mas_.ncoarse * mas_.tile_elems * esz + 2.0 * n * 8 +
                             (double)pat_.nb * (1 + 4);
    const double vb = p_.mixed ? 4.0 : 8.0;  // operator value bytes of the residual SpMV
    // r, x, y in FP32 in mixed precision, FP64 otherwise
    const double res_bytes = (double)nnzb * (bd * bd * vb + 4) + (pat_.nb + 1) * 4.0 + (p_.mixed ? 12.0 : 24.0) * n;
    const double mas0_bytes = inv0_bytes + 2.0 * n * 8 + (double)pat_.nb * 5;
    switch (kind) {
    case 0: *bytes = spmv_bytes; break;
    case 1: *bytes = mas_bytes; break;
    case 4: *bytes = mas0_bytes; break;
    case 5: *bytes = res_bytes; break;
    case 6: *bytes = spmv_bytes + 8.0 * n; break;  // + p for p.Ap
    default: *bytes = 0; break;
    }
}

}  // namespace lss
