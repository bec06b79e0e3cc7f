// FP64 multifrontal factor of the large stiff subdomains.
//
// The reference factors each stiff subdomain with cuDSS (batched sparse
// LDL^T; GPUHybrid.cu:1075-1196 extraction, :1248-1249 analysis and
// factorization) and applies A_SS^-1 by its triangular solves
// (dss_precond_iter, GPUHybrid.cu:544-675).  Here a subdomain above the dense
// size gets a nested-dissection elimination tree (host, symbolic); every tree
// node ("front") is a dense matrix over its own variables (a separator, or a
// leaf) and the later variables they couple to (its boundary).  On the GPU,
// level by level of the tree: the original entries and the children's update
// matrices are summed into the front (extend-add, children in a fixed order),
// and the front's own pivots are swept (the symmetric Gauss-Jordan sweep of
// the MAS inverses, applied to the leading pivots only), which leaves
//     [ -F11^-1        F11^-1 F12 ]
//     [ F21 F11^-1     F22 - F21 F11^-1 F12 ]
// in place: the pivot block's inverse, the coupling P = F21 F11^-1 and the
// Schur complement U that the parent sums in.  The factor is FP64 (the
// batched 16-right-hand-side solve applies it as double-float pairs).  The
// solve is one GEMV per front and direction:
//     forward (leaves first):  c = w_bnd - P w_own      (passed to the parent)
//     backward (root first):   x_own = F11^-1 (w_own - F12 x_bnd)
// where w_own holds the right-hand side plus the children's contributions.
// All sums run in a fixed order: the factor and the solve are deterministic.
#pragma once

#include <cstdint>
#include <vector>

#include "kernels.hpp"
#include "lss_common.hpp"

namespace lss {

// Fronts up to this size are swept by one CTA in shared memory.
constexpr int MF_SMEM_F = 160;

// Host symbolic structure of all large subdomains together.  Positions
// (elimination order) are global over the subdomains; the variables of a
// subtree occupy a contiguous range of positions and a front's own variables
// are the last of its subtree.
struct MfSymbolic {
    int32_t nfront = 0, npos = 0, levels = 0;
    std::vector<int32_t> p0, s, u, height;     // per front
    std::vector<int64_t> foff;                 // per front: element offset of its f x f storage
    std::vector<int32_t> woff;                 // per front: offset of its solve vector (f entries)
    std::vector<int32_t> bnd_off, bnd_pos;     // boundary positions per front (ascending)
    std::vector<int32_t> child_off, child;     // children per front (ascending front ids)
    std::vector<int32_t> ea_map;               // per front (as a child): index in the parent front of
                                               // each boundary entry (aligned with bnd_pos)
    std::vector<int32_t> front_of_pos;         // per position
    std::vector<int32_t> pos2j;                // per position: index into the stiff DOF list
    std::vector<int32_t> j2pos;                // per large-subdomain DOF (j - j_base): its position
    int32_t j_base = 0;                        // first stiff-DOF index of the large subdomains
    int64_t elems = 0;                         // front storage (doubles)
    int64_t welems = 0;                        // solve vectors (doubles)
    int32_t max_f = 0, max_s = 0;
    double fmas = 0.0;                         // FMAs of the numeric factorization
};

// dofs: the stiff DOF list (permuted scalar ids, ascending within each
// subdomain); off: subdomain offsets into it; the subdomains k >= first_large
// get the multifrontal factor.  rows / cols: the permuted block pattern.
MfSymbolic mf_symbolic(const std::vector<int32_t> &dofs, const std::vector<int32_t> &off, int32_t first_large,
                       const std::vector<int32_t> &rows, const std::vector<int32_t> &cols, int bd);

// CTA work list: CTAs [prefix[i], prefix[i+1]) of a launch belong to front[i].
struct MfWork {
    int32_t count = 0;
    int64_t ctas = 0;
    const int32_t *front = nullptr;
    const int64_t *prefix = nullptr;
    const int32_t *cta_item = nullptr;  // optional: per CTA its index i (saves the search)
};

// The device side: symbolic arrays, front storage, solve vectors, and the
// per-level work lists of every kernel.
class MfFactor {
public:
    void setup(const MfSymbolic &sym, cudaStream_t s);  // uploads the plan
    bool empty() const { return sym_.nfront == 0; }
    // numeric factorization (values of A in the permuted operator)
    void factorize(const BsrDev &A, const StiffDev &S, int *bad, cudaStream_t s);
    // z[d] += (A_SS^-1 t)_d over the large subdomains, t = S.t
    void solve(const StiffDev &S, double *z, float *z32, float *z_lo, const int *done, cudaStream_t s);
    // z[d][k] += (A_SS^-1 t)[d][k] for 16 right-hand sides at once: t is
    // [stiff DOF][16] (FP64), z a [row][16] double-float pair vector.  Fronts
    // of a system with sys_done[front_sys[N]] set are skipped.
    void solve_batch(const StiffDev &S, const double *t, float2 *z, const int *sys_done, const int32_t *front_sys,
                     cudaStream_t s);
    // the fronts as double-float pairs for solve_batch (after the fronts are final)
    void make_pairs(cudaStream_t s);
    const MfSymbolic &symbolic() const { return sym_; }
    // device front storage (f x f per front, foff offsets), for merging factors
    const double *fronts() const { return d_F_.data(); }
    double *fronts_mut() { return d_F_.data(); }
    int64_t bytes() const;

private:
    struct Level {
        MfWork ea, small, diag, panel, update, write, mirror, fasm_nr, fwd_nr, bwd_nr, fasm1;
        int32_t max_s_large = 0;
    };
    MfSymbolic sym_;
    std::vector<Level> levels_;
    DBuf<int32_t> d_i32_;  // symbolic arrays and work-list fronts
    DBuf<int64_t> d_i64_;  // front offsets and work-list prefixes
    DBuf<double> d_F_, d_w_, d_x_, d_P_, d_D_;
    DBuf<float2> d_wb_, d_xb_;  // solve vectors of the batched solve (double-float pairs)
    DBuf<float2> d_Fp_;         // fronts as (hi, lo) FP32 pairs, for the batched solve
    DBuf<float2> d_nrpart_;     // batched solve: per GEMV CTA partial sums of split fronts
    DBuf<unsigned> d_nrcnt_;    // arrival counters of split fronts (both solves)
    DBuf<double> d_part1_;      // single right-hand-side solve: per GEMV CTA partial sums
    const int32_t *p0_ = nullptr, *s_ = nullptr, *u_ = nullptr, *woff_ = nullptr, *bnd_off_ = nullptr,
                  *bnd_pos_ = nullptr, *child_off_ = nullptr, *child_ = nullptr, *ea_map_ = nullptr,
                  *front_of_pos_ = nullptr, *pos2j_ = nullptr, *j2pos_ = nullptr, *poff_ = nullptr;
    const int64_t *foff_ = nullptr;
    const int32_t *gptr_ = nullptr, *gsrc_ = nullptr;  // extend-add gather lists (batched solve)
};

}  // namespace lss
