// Shared host-side definitions of the GB300 hybrid solver: status codes,
// errors, device buffers, parameters.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/lss.h"

namespace lss {

// Exception carrying a C-ABI status code; the C-ABI converts it to a return value.
struct Error : std::runtime_error {
    lss_status code;
    Error(lss_status c, const std::string &m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(lss_status c, const std::string &m) { throw Error(c, m); }

inline void cuda_check(cudaError_t e, const char *what, const char *file, int line)
{
    if (e == cudaSuccess) return;
    std::string msg = std::string(what) + " failed at " + file + ":" + std::to_string(line) + ": " +
                      cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) {
        size_t fr = 0, tot = 0;
        cudaGetLastError();
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess)
            msg += " [free " + std::to_string(fr >> 20) + " MiB of " + std::to_string(tot >> 20) + " MiB]";
        throw Error(LSS_ERR_OOM, msg);
    }
    throw Error(LSS_ERR_CUDA, msg);
}
// Kernel launch bookkeeping: launches issued by launcher functions plus the
// kernel nodes of replayed CUDA graphs (reported by get_info); atomic because
// batched solves drive several solvers from host threads at once.
std::atomic<unsigned long long> &launch_count();
#define LSS_CUDA(call) ::lss::cuda_check((call), #call, __FILE__, __LINE__)
#define LSS_LAUNCH_CHECK() \
    (::lss::launch_count()++, ::lss::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__))

// Makes `dev` current for a scope and restores the caller's device after.
struct CudaDeviceGuard {
    int saved = -1;
    explicit CudaDeviceGuard(int dev)
    {
        if (cudaGetDevice(&saved) != cudaSuccess) {
            cudaGetLastError();
            saved = -1;
        }
        if (saved != dev) cuda_check(cudaSetDevice(dev), "cudaSetDevice", __FILE__, __LINE__);
    }
    ~CudaDeviceGuard()
    {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

// Optional allocation cap for fault testing of the OOM path: at most
// alloc_cap_bytes() more bytes than were live when the cap was set
// (alloc_cap_base()); 0 = no cap.  Atomic: the batched entry points allocate
// from several host threads at once.
std::atomic<size_t> &alloc_cap_bytes();
std::atomic<size_t> &alloc_cap_base();
std::atomic<size_t> &alloc_live_bytes();

// Books `bytes` against the live total before a cudaMalloc; the check against
// the cap and the addition are one compare-and-swap, so concurrent
// allocations can neither slip past the cap nor lose an update.
inline void alloc_reserve(size_t bytes)
{
    std::atomic<size_t> &live = alloc_live_bytes();
    size_t cur = live.load();
    for (;;) {
        const size_t cap = alloc_cap_bytes().load();
        if (cap && cur + bytes > alloc_cap_base().load() + cap)
            fail(LSS_ERR_OOM, "device allocation of " + std::to_string(bytes) +
                                  " bytes exceeds the configured memory cap");
        if (live.compare_exchange_weak(cur, cur + bytes)) return;
    }
}
inline void alloc_unreserve(size_t bytes) { alloc_live_bytes().fetch_sub(bytes); }

// Owning device allocation (cudaMalloc), move-only.
template <typename T>
class DBuf {
public:
    DBuf() = default;
    explicit DBuf(size_t n) { resize(n); }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    DBuf &operator=(DBuf &&o) noexcept
    {
        if (this != &o) { release(); p_ = o.p_; n_ = o.n_; o.p_ = nullptr; o.n_ = 0; }
        return *this;
    }
    ~DBuf() { release(); }

    void resize(size_t n)
    {
        if (n == n_) return;
        release();
        if (n == 0) return;
        const size_t bytes = n * sizeof(T);
        alloc_reserve(bytes);
        const cudaError_t e = cudaMalloc(&p_, bytes);
        if (e != cudaSuccess) {
            p_ = nullptr;
            alloc_unreserve(bytes);
            cuda_check(e, "cudaMalloc", __FILE__, __LINE__);
        }
        n_ = n;
    }
    void release()
    {
        if (p_) {
            cudaFree(p_);
            alloc_unreserve(n_ * sizeof(T));
        }
        p_ = nullptr;
        n_ = 0;
    }
    void upload(const T *h, size_t n, cudaStream_t s)
    {
        resize(n);
        if (n) LSS_CUDA(cudaMemcpyAsync(p_, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T> &h, cudaStream_t s) { upload(h.data(), h.size(), s); }
    void zero(cudaStream_t s)
    {
        if (n_) LSS_CUDA(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s));
    }
    std::vector<T> download(cudaStream_t s) const
    {
        std::vector<T> h(n_);
        if (n_) {
            LSS_CUDA(cudaMemcpyAsync(h.data(), p_, n_ * sizeof(T), cudaMemcpyDeviceToHost, s));
            LSS_CUDA(cudaStreamSynchronize(s));
        }
        return h;
    }
    T *data() { return p_; }
    const T *data() const { return p_; }
    size_t size() const { return n_; }
    size_t bytes() const { return n_ * sizeof(T); }
    bool empty() const { return n_ == 0; }

private:
    T *p_ = nullptr;
    size_t n_ = 0;
};

// Pinned host staging buffer (grows, never shrinks).
class PinnedBuf {
public:
    ~PinnedBuf() { if (p_) cudaFreeHost(p_); }
    void *get(size_t bytes)
    {
        if (bytes > cap_) {
            if (p_) cudaFreeHost(p_);
            p_ = nullptr;
            LSS_CUDA(cudaMallocHost(&p_, bytes));
            cap_ = bytes;
        }
        return p_;
    }

private:
    void *p_ = nullptr;
    size_t cap_ = 0;
};

// Solver parameters.  The first block mirrors the reference's GPUHybrid keys
// (GPUHybrid.hpp:72-93, linear-solver-spec.json:495-519, 646-747) with the
// spec defaults; the second block is this implementation's "gb300" sub-object.
struct Params {
    int max_iter = 10000;
    double rel_tol = 1e-10;
    double abs_tol = 0.0;
    int block_size = 1;
    double theta = 0.5;  // accepted, unused (no strength threshold in MAS)
    bool do_hybrid = true;
    bool select_l1 = true;
    double jump_threshold = 100.0;
    double gmm_tol = 1e-3;
    int max_gmm_iterations = 20;
    double cond_threshold = 100.0;
    bool decompose = true;
    int min_sub = 1;
    int max_sub = 10000000;
    bool expand = true;
    int max_dense_size = 0;         // accepted; every subdomain uses the dense factor
    bool float_subdomains = false;  // store stiff-block inverses in FP32

    // "gb300" extension
    bool mixed = false;             // FP32 MAS (+ FP32 operator inside the preconditioner)
    int outer_spmv = 0;             // PCG's A p: 0 auto (df32 iff mixed), 1 FP64, 2 df32 (FP32-pipe double-float)
    int precond_residual = 0;       // mixed r - A z: 0 auto (df32 on stiff rows), 1 FP32, 2 df32 everywhere
    bool mas_bf16_offdiag = false;  // mixed: BF16 storage of the level-0 off-diagonal inverse tiles
    // MASSolver's bad-DOF selections (linear-solver-spec.json "/MAS/bad_dof_*"
    // keys and defaults) in place of GPUHybrid's GMM + post-processing
    int bad_dof_strategy = 0;       // BadDofStrategy: 0 GPUHybrid, 1 elbow, 2 kmean, 3 gmm
    double kmeans_search_fraction = 0.2, kmeans_jump_threshold = 10.0;
    int kmeans_max_iterations = 32, kmeans_expand_neighbors = 128;
    double mas_gmm_jump_threshold = 10.0, mas_gmm_tol = 1e-3;
    int mas_gmm_max_iterations = 20, mas_gmm_expand_neighbors = 16;
    int bad_dof_max_block = 20000;  // components above this (dense inverse) are dropped
    bool multiplicative = true;     // GPUHybrid composition; false = MASSolver additive form
    int max_coarse_levels = 4;      // MAS_MAX_COARSE_LEVEL (MASPreconditioner.hpp:11); <= 6
    double mas_damping = 0.0;       // omega of MAS in the multiplicative form; <= 0: automatic
    int omega_iters = 20;           // PCG-Lanczos steps of the automatic estimate
    double omega_factor = 1.5;      // omega = omega_factor / lambda_max(MAS A)
    int check_every = 8;            // PCG iterations per host convergence poll
    int max_refinements = 2;        // true-residual restarts when the recurrence drifted
    int device = 0;
    int partition_threads = 0;      // 0 = hardware concurrency (max 16)
    bool use_graphs = true;         // capture the PCG iteration chunk in a CUDA graph
    int spmv_lanes = 0;             // lanes per block row in SpMV; 0 = autotune
    size_t memory_cap_bytes = 0;    // fault testing: cap device allocations
};

Params parse_params(const char *json, const Params &base);

}  // namespace lss
