// Batched solves: many factorized systems of uneven size, each with BK
// right-hand sides, advanced together by one PCG whose every step is a single
// launch over all systems and all right-hand sides.
//
// The reference solves one system per call (GPUHybrid::solve,
// GPUHybrid.cu:342-399, PCG :1413-1512); a batch runs exactly that PCG for
// every (system, right-hand side) lane -- its own alpha, beta, gamma and
// stopping test -- but the operator, the MAS inverses and the stiff factors
// of a system are read once per iteration for all BK right-hand sides.  The
// iterations run on a correction in double-float; the solution accumulates in
// FP64 at every restart, where the residual b - A x is recomputed in FP64
// (iterative refinement), so the attainable accuracy is FP64's.
//
// The systems are factorized one by one (each keeps its own selection,
// partition, MAS hierarchy, damping and stiff factor) and then merged into one
// block-diagonal device image: the block rows, MAS banks and coarse items of
// system s follow those of s - 1 (coarse levels padded to whole banks, so no
// bank mixes two systems), the dense stiff inverses and the multifrontal
// fronts are concatenated.  Vectors are stored RHS-interleaved, [row][BK].
// Every reduction is segmented by system over fixed "chunks" of partitions
// and finished by the last CTA of the system to arrive, in chunk order: the
// results do not depend on scheduling.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "kernels.hpp"
#include "lss_common.hpp"
#include "multifrontal.hpp"

namespace lss {

constexpr int BK = 16;           // right-hand sides per system in a batch
constexpr int BATCH_CHUNK = 8;   // MAS partitions (<= 32 block rows each) per chunk

class HybridSolver;

// Per-lane PCG state, lane = system * BK + rhs.
struct BatchLane {
    double bb, gamma, alpha, beta, pAp, rr, rel_eps, abs_eps;
    int iter, done, max_iter, pad;
};

// Device view of the merged batch (BD = 3).
struct BatchDev {
    int32_t nsys = 0, nb = 0, nchunk = 0;
    int64_t n = 0;
    // operator (row-sliced BSR as in spmv.cuh): rows, cols, and three value copies
    const int32_t *rows = nullptr, *cols = nullptr;
    const double *vals = nullptr;
    const float *vals32 = nullptr;
    const float2 *vals_df = nullptr;
    const uint8_t *precise = nullptr;   // block rows whose preconditioner residual runs in double-float
    // chunks: chunk c = parts [chunk_p0[c], chunk_p0[c+1]) of system chunk_sys[c]
    const int32_t *chunk_sys = nullptr, *chunk_p0 = nullptr;
    const int32_t *sys_chunk0 = nullptr;  // nsys + 1
    const int32_t *part_off = nullptr;    // merged MAS parts (nparts + 1), block-row offsets
    const double *omega = nullptr;        // per system: damping of MAS in the multiplicative form
    BatchLane *lane = nullptr;            // nsys * BK
    const int *sys_done = nullptr;        // per system: every lane stopped
    int *err = nullptr;                   // != 0: a bulk copy did not arrive (sys_done[nsys])
    double *partials = nullptr;           // nchunk * BK * 2
    unsigned *counters = nullptr;         // nsys
};

// Merged MAS levels (FP32 inverses).  Level-l items of system s start at a
// multiple of 32 (whole banks); a bank whose system has no level l + 1 has
// ccnt = 0.
struct BatchMas {
    MasDev m;                              // merged level sizes, maps and offsets (pointers into own buffers)
    const float *inv0 = nullptr, *invc = nullptr;  // inv0: full 96 x 96 matrices; invc: stored diagonals
    float *v = nullptr, *u = nullptr;      // level vectors, [item * BD + c][BK]
};

struct BatchStiff {
    StiffDev S;                            // dense subdomains (j < ndof_dense) + multifrontal DOFs
    double *t = nullptr;                   // [ndof][BK]
};

namespace bk {
// a system's user vectors (n_s x BK column-major) and where its rows go
struct ScatterSys {
    const double *src;
    double *dst;
    int32_t nb, row0;     // block rows of the system, first merged block row
    const int32_t *perm;  // the system's partition permutation (old block -> new)
};
void launch_spmm_alpha(const BatchDev &B, const float2 *p, float2 *ap, cudaStream_t s);
void launch_update_xr(const BatchDev &B, float2 *x, float2 *r, const float2 *p, const float2 *ap, cudaStream_t s);
void launch_update_p(const BatchDev &B, float2 *p, const float2 *z, cudaStream_t s);
void launch_copy_pairs(const BatchDev &B, float2 *dst, const float2 *src, cudaStream_t s);
// mode 0: r = b - A x (and rr); mode 1: rr only; x in FP64
void launch_residual64(const BatchDev &B, const double *b, const double *x, float2 *r, int mode, double *rr,
                       cudaStream_t s);
// xt += x (pairs), x = 0
void launch_fold(const BatchDev &B, double *xt, float2 *x, cudaStream_t s);
void launch_lane_norms(const BatchDev &B, const double *b, double *bb, cudaStream_t s);
// z = omega M x (acc: z += ...); x as pairs (xin_pair) or FP32 (xin32); dot 1 / 2: gamma (and beta) = r.z
void launch_mas(const BatchDev &B, const BatchMas &M, const float2 *xin_pair, const float *xin32, float2 *z, bool acc,
                int dot, const float2 *rdot, cudaStream_t s);
void launch_residual32(const BatchDev &B, const float2 *r, const float2 *z, float *w, cudaStream_t s);
// the level-0 banks' stored diagonals expanded into full 96 x 96 column-major matrices
void launch_expand_banks(const float *tiles, float *full, int64_t nbank, cudaStream_t s);
// t = r_S - (A z)_S over every stiff DOF; z_S += Inv t over the dense subdomains
void launch_stiff(const BatchDev &B, const StiffDev &S, const float2 *r, const float2 *z_in, double *t, float2 *z,
                  cudaStream_t s);
// user column-major vectors (src) -> [row][BK] FP64 (dst), and back (dst of the table)
void launch_to_batch(const ScatterSys *sys, int nsys, const int64_t *prefix, int64_t total, double *dst,
                     cudaStream_t s);
void launch_from_batch(const ScatterSys *sys, int nsys, const int64_t *prefix, int64_t total, const double *src,
                       cudaStream_t s);
// x = 0 for the lanes with a zero right-hand side (GPUHybrid.cu:1428-1439)
void launch_zero_done_lanes(const BatchDev &B, double *x, cudaStream_t s);
}  // namespace bk

class BatchSolver {
public:
    // systems: factorized solvers (block size 3, mixed precision, multiplicative
    // GPUHybrid composition), each used by this batch only
    BatchSolver(std::vector<HybridSolver *> systems, int device);
    ~BatchSolver();
    BatchSolver(const BatchSolver &) = delete;
    BatchSolver &operator=(const BatchSolver &) = delete;

    // factorize every system with values in device memory (host-thread pool),
    // then merge them into the batch image
    void factorize_device(const double *const *d_values, int threads);
    // d_b[s], d_x[s]: n_s x BK column-major (leading dimension n_s); x is the
    // initial guess on entry.  iterations (optional): nsys * BK.
    void solve_device(const double *const *d_b, double *const *d_x, int32_t *iterations);
    std::string info_json() const;
    int device() const { return device_; }

private:
    void merge();
    void iteration();
    void precond(int dot_mode);
    void launch_chunk(int iters);
    void invalidate_graph();

    std::vector<HybridSolver *> sys_;
    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    bool merged_ = false;
    struct Impl;
    std::unique_ptr<Impl> d_;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_iters_ = 0;
    size_t graph_nodes_ = 0;
    std::vector<int32_t> last_iters_;
    double last_solve_s_ = 0.0, last_merge_s_ = 0.0, last_factorize_s_ = 0.0;
    int last_refinements_ = 0;
};

}  // namespace lss
