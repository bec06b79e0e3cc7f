// Host side of the batched PCG (batch.hpp): merging factorized systems into
// one block-diagonal image and driving the iterations as CUDA-graph chunks.
#include "batch.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <sstream>
#include <thread>

#include "solver.hpp"

namespace lss {


namespace {
using clk = std::chrono::steady_clock;
double secs(clk::time_point t0) { return std::chrono::duration<double>(clk::now() - t0).count(); }

template <typename T>
void append(std::vector<T> &dst, const std::vector<T> &src, T add = T(0))
{
    const size_t at = dst.size();
    dst.resize(at + src.size());
    for (size_t i = 0; i < src.size(); ++i) dst[at + i] = src[i] + add;
}
}  // namespace

struct BatchSolver::Impl {
    BatchDev B;
    BatchMas M;
    BatchStiff St;
    MfFactor mf;
    // operator and chunks
    DBuf<int32_t> rows, cols, chunk_sys, chunk_p0, sys_chunk0, part_off;
    DBuf<double> vals, omega, partials;
    DBuf<float> vals32;
    DBuf<float2> vals_df;
    DBuf<uint8_t> precise;
    DBuf<BatchLane> lane;
    DBuf<int> sys_done;
    DBuf<unsigned> counters;
    // MAS
    DBuf<uint8_t> key0, ccnt0;
    DBuf<int32_t> cbase0;
    std::vector<DBuf<uint8_t>> key, ccnt;
    std::vector<DBuf<int32_t>> cbase;
    DBuf<float> inv0, invc, v, u;
    DBuf<float> inv0x;  // level-0 banks as full 96 x 96 matrices (the level-0 apply reads these)
    // stiff
    DBuf<int32_t> sdofs, ssub, soff, front_sys;
    DBuf<int64_t> sinvoff;
    DBuf<double> sinv, t;
    // vectors [n][BK]
    DBuf<double> b, rr, xt;  // right-hand sides, lane sums, the solution (FP64)
    DBuf<float2> x, r, p, z, ap;
    DBuf<float> w;
    // host
    std::vector<int32_t> row0, part0, nb_sys;
    std::vector<BatchLane> h_lane;
    std::vector<int> h_done;
    std::vector<double> h_rr;
    int32_t nparts = 0;
    DBuf<bk::ScatterSys> scat;
    DBuf<int64_t> scat_prefix;
};

BatchSolver::BatchSolver(std::vector<HybridSolver *> systems, int device)
    : sys_(std::move(systems)), device_(device), d_(new Impl)
{
    if (sys_.empty()) fail(LSS_ERR_INVALID_ARGUMENT, "a batch needs at least one system");
    for (size_t i = 0; i < sys_.size(); ++i)
        for (size_t j = i + 1; j < sys_.size(); ++j)
            if (sys_[i] == sys_[j]) fail(LSS_ERR_INVALID_ARGUMENT, "batched systems must be distinct solver objects");
    for (HybridSolver *s : sys_) {
        if (s->device() != device) fail(LSS_ERR_INVALID_ARGUMENT, "batched systems must share one device");
        if (s->p_.block_size != 3 || !s->p_.mixed || !s->p_.multiplicative || !s->df32() || !s->p_.do_hybrid ||
            s->p_.bad_dof_strategy != 0)
            fail(LSS_ERR_UNSUPPORTED, "the batched PCG takes block size 3, mixed precision, the GPUHybrid "
                                      "selection and the multiplicative composition");
    }
    LSS_CUDA(cudaSetDevice(device_));
    LSS_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
}

BatchSolver::~BatchSolver()
{
    invalidate_graph();
    if (stream_) {
        cudaStreamSynchronize(stream_);
        cudaStreamDestroy(stream_);
    }
}

void BatchSolver::invalidate_graph()
{
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    graph_exec_ = nullptr;
    graph_iters_ = 0;
}

void BatchSolver::factorize_device(const double *const *d_values, int threads)
{
    auto t0 = clk::now();
    const int32_t count = (int32_t)sys_.size();
    const int nthreads = threads > 0 ? std::min<int>(threads, count) : count;
    std::atomic<int32_t> next{0};
    std::mutex mu;
    std::string first;
    lss_status code = LSS_OK;
    auto worker = [&]() {
        for (;;) {
            const int32_t s = next.fetch_add(1);
            if (s >= count) return;
            try {
                LSS_CUDA(cudaSetDevice(device_));
                sys_[s]->factorize_device(d_values[s], nullptr);
            } catch (const Error &e) {
                std::lock_guard<std::mutex> lock(mu);
                if (code == LSS_OK) {
                    code = e.code;
                    first = "system " + std::to_string(s) + ": " + e.what();
                }
            } catch (const std::exception &e) {
                std::lock_guard<std::mutex> lock(mu);
                if (code == LSS_OK) {
                    code = LSS_ERR_INTERNAL;
                    first = "system " + std::to_string(s) + ": " + e.what();
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto &th : pool) th.join();
    LSS_CUDA(cudaSetDevice(device_));
    if (code != LSS_OK) fail(code, first);
    last_factorize_s_ = secs(t0);
    auto t1 = clk::now();
    merge();
    last_merge_s_ = secs(t1);
}

// ------------------------------------------------------------------ merge

void BatchSolver::merge()
{
    merged_ = false;
    invalidate_graph();
    Impl &D = *d_;
    const int32_t ns = (int32_t)sys_.size();
    constexpr int BDIM = 3;
    // ---- operator, parts, chunks
    std::vector<int32_t> rows{0}, cols, part_off{0}, chunk_sys, chunk_p0, sys_chunk0{0};
    std::vector<uint8_t> precise;
    std::vector<double> omega;
    D.row0.assign(ns, 0);
    D.part0.assign(ns, 0);
    D.nb_sys.assign(ns, 0);
    int32_t nb = 0, np = 0;
    int64_t nnzb = 0;
    bool any_precise = false;
    for (int32_t s = 0; s < ns; ++s) {
        const HybridSolver &H = *sys_[s];
        const Pattern &P = H.pat_;
        D.row0[s] = nb;
        D.part0[s] = np;
        D.nb_sys[s] = P.nb;
        for (int32_t i = 0; i < P.nb; ++i) rows.push_back((int32_t)(nnzb + P.rows[i + 1]));
        append(cols, P.cols, nb);
        const auto &po = P.part.part_offsets;
        const int32_t nps = (int32_t)po.size() - 1;
        for (int32_t q = 1; q <= nps; ++q) part_off.push_back(nb + po[q]);
        for (int32_t q = 0; q < nps; q += BATCH_CHUNK) {
            chunk_sys.push_back(s);
            chunk_p0.push_back(np + q);
        }
        sys_chunk0.push_back((int32_t)chunk_sys.size());
        if (H.h_precise_.size() == (size_t)P.nb) {
            precise.insert(precise.end(), H.h_precise_.begin(), H.h_precise_.end());
            any_precise = true;
        } else {
            precise.insert(precise.end(), P.nb, 0);
        }
        omega.push_back(H.omega_);
        nb += P.nb;
        np += nps;
        nnzb += P.rows.back();
    }
    chunk_p0.push_back(np);
    D.nparts = np;
    const cudaStream_t st = stream_;
    D.rows.upload(rows, st);
    D.cols.upload(cols, st);
    D.part_off.upload(part_off, st);
    D.chunk_sys.upload(chunk_sys, st);
    D.chunk_p0.upload(chunk_p0, st);
    D.sys_chunk0.upload(sys_chunk0, st);
    D.omega.upload(omega, st);
    if (any_precise) D.precise.upload(precise, st);
    else D.precise.release();
    D.vals.resize(nnzb * 9);
    D.vals32.resize(nnzb * 9);
    D.vals_df.resize(nnzb * 9);
    {
        int64_t at = 0;
        for (int32_t s = 0; s < ns; ++s) {
            const HybridSolver &H = *sys_[s];
            const int64_t cnt = (int64_t)H.pat_.rows.back() * 9;
            LSS_CUDA(cudaMemcpyAsync(D.vals.data() + at, H.d_vals_.data(), cnt * 8, cudaMemcpyDeviceToDevice, st));
            LSS_CUDA(cudaMemcpyAsync(D.vals32.data() + at, H.d_vals32_.data(), cnt * 4, cudaMemcpyDeviceToDevice, st));
            LSS_CUDA(cudaMemcpyAsync(D.vals_df.data() + at, H.d_vals_df_.data(), cnt * 8, cudaMemcpyDeviceToDevice, st));
            at += cnt;
        }
    }
    const int32_t nchunk = (int32_t)chunk_sys.size();
    D.partials.resize((size_t)std::max(nchunk, 1) * BK * 2);
    D.counters.resize(ns);
    D.counters.zero(st);
    D.lane.resize((size_t)ns * BK);
    D.sys_done.resize((size_t)ns + 1);  // + the kernels' error status
    D.rr.resize((size_t)ns * BK);

    // ---- MAS: levels padded to whole banks per system
    int L = 1;
    for (HybridSolver *H : sys_) L = std::max(L, H->cs_.L);
    if (L > MAS_MAXL) fail(LSS_ERR_INTERNAL, "MAS levels beyond the batch's limit");
    std::vector<std::vector<int32_t>> bank_off(L, std::vector<int32_t>(ns + 1, 0));
    for (int l = 1; l < L; ++l)
        for (int32_t s = 0; s < ns; ++s)
            bank_off[l][s + 1] = bank_off[l][s] + (l < sys_[s]->cs_.L ? sys_[s]->cs_.nbanks[l] : 0);
    std::vector<uint8_t> key0, ccnt0;
    std::vector<int32_t> cbase0;
    for (int32_t s = 0; s < ns; ++s) {
        const CoarseSpace &cs = sys_[s]->cs_;
        append(key0, cs.key0);
        if (cs.L > 1) {
            append(ccnt0, cs.ccnt0);
            append(cbase0, cs.cbase0, 32 * bank_off[1][s]);
        } else {
            ccnt0.insert(ccnt0.end(), cs.ccnt0.size(), 0);
            cbase0.insert(cbase0.end(), cs.cbase0.size(), 0);
        }
    }
    D.key0.upload(key0, st);
    D.ccnt0.upload(ccnt0, st);
    D.cbase0.upload(cbase0, st);
    D.key.clear();
    D.ccnt.clear();
    D.cbase.clear();
    D.key.resize(L);
    D.ccnt.resize(L);
    D.cbase.resize(L);
    MasDev &m = D.M.m;
    m = MasDev();
    m.L = L;
    m.bd = BDIM;
    m.nb = nb;
    m.nparts = np;
    m.part_off = D.part_off.data();
    m.key0 = D.key0.data();
    m.cbase0 = D.cbase0.data();
    m.ccnt0 = D.ccnt0.data();
    m.nbanks[0] = np;
    m.tile_elems = mas_tile_elems(BDIM);
    int64_t voff = 0;
    int32_t boff = 0;
    for (int l = 1; l < L; ++l) {
        m.nbanks[l] = bank_off[l][ns];
        m.nitems[l] = 32 * bank_off[l][ns];
        m.voff[l] = voff;
        voff += (int64_t)m.nitems[l] * BDIM;
        m.boff[l] = boff;
        boff += m.nbanks[l];
        if (l + 1 < L) {
            std::vector<uint8_t> key, ccnt;
            std::vector<int32_t> cbase;
            for (int32_t s = 0; s < ns; ++s) {
                const CoarseSpace &cs = sys_[s]->cs_;
                if (l >= cs.L) continue;
                const int32_t nbk = cs.nbanks[l];
                if (l + 1 < cs.L) {
                    std::vector<uint8_t> kk(cs.key[l].begin(), cs.key[l].begin() + (size_t)nbk * 32);
                    append(key, kk);
                    append(ccnt, cs.ccnt[l]);
                    append(cbase, cs.cbase[l], 32 * bank_off[l + 1][s]);
                } else {  // the system's top level: no parent aggregates
                    key.insert(key.end(), (size_t)nbk * 32, 0);
                    ccnt.insert(ccnt.end(), nbk, 0);
                    cbase.insert(cbase.end(), nbk, 0);
                }
            }
            D.key[l].upload(key, st);
            D.ccnt[l].upload(ccnt, st);
            D.cbase[l].upload(cbase, st);
            m.key[l] = D.key[l].data();
            m.ccnt[l] = D.ccnt[l].data();
            m.cbase[l] = D.cbase[l].data();
        }
    }
    m.ncoarse = boff;
    m.level_elems = voff;
    const int64_t te = m.tile_elems;
    D.inv0.resize((size_t)np * te);
    D.invc.resize((size_t)std::max<int32_t>(boff, 1) * te);
    for (int32_t s = 0; s < ns; ++s) {
        const HybridSolver &H = *sys_[s];
        if (H.mas_.bank_bytes0 > 0) fail(LSS_ERR_UNSUPPORTED, "the batched PCG takes FP32 MAS tiles");
        const int32_t nps = H.mas_.nparts;
        LSS_CUDA(cudaMemcpyAsync(D.inv0.data() + (int64_t)D.part0[s] * te, H.d_inv0_.data(), (size_t)nps * te * 4,
                                 cudaMemcpyDeviceToDevice, st));
        for (int l = 1; l < H.cs_.L; ++l) {
            const int32_t nbk = H.cs_.nbanks[l];
            if (nbk == 0) continue;
            const float *src = reinterpret_cast<const float *>(H.d_invc_.data()) + (int64_t)H.mas_.boff[l] * te;
            float *dst = D.invc.data() + (int64_t)(m.boff[l] + bank_off[l][s]) * te;
            LSS_CUDA(cudaMemcpyAsync(dst, src, (size_t)nbk * te * 4, cudaMemcpyDeviceToDevice, st));
        }
    }
    D.v.resize((size_t)std::max<int64_t>(voff, 1) * BK);
    D.u.resize((size_t)std::max<int64_t>(voff, 1) * BK);
    D.v.zero(st);
    D.u.zero(st);
    // level-0 banks expanded once into full matrices: the apply then copies
    // them into shared memory as they are, instead of expanding the stored
    // diagonals on every apply
    D.inv0x.resize((size_t)np * (32 * BDIM) * (32 * BDIM));
    bk::launch_expand_banks(D.inv0.data(), D.inv0x.data(), np, st);
    LSS_CUDA(cudaStreamSynchronize(st));
    D.inv0.release();
    D.M.inv0 = D.inv0x.data();
    D.M.invc = D.invc.data();
    D.M.v = D.v.data();
    D.M.u = D.u.data();

    // ---- stiff blocks: every system's dense subdomains, then every system's multifrontal ones
    std::vector<int32_t> sdofs, ssub, soff{0}, front_sys;
    std::vector<int64_t> sinvoff;
    int32_t nsub = 0;
    int64_t inv_at = 0;
    for (int pass = 0; pass < 2; ++pass)
        for (int32_t s = 0; s < ns; ++s) {
            const HybridSolver &H = *sys_[s];
            const int32_t nss = (int32_t)H.h_soff_.size() - 1;
            const int32_t k0 = pass == 0 ? 0 : H.ndense_, k1 = pass == 0 ? H.ndense_ : nss;
            for (int32_t k = k0; k < k1; ++k) {
                for (int32_t j = H.h_soff_[k]; j < H.h_soff_[k + 1]; ++j) {
                    sdofs.push_back(H.h_sdofs_[j] + D.row0[s] * BDIM);
                    ssub.push_back(nsub);
                }
                soff.push_back((int32_t)sdofs.size());
                sinvoff.push_back(pass == 0 ? inv_at + H.h_sinvoff_[k] : 0);
                ++nsub;
            }
            if (pass == 0) inv_at += H.inv_total_;
        }
    const int32_t ndense_dofs = [&]() {
        int32_t c = 0;
        for (HybridSolver *H : sys_) c += H->h_soff_[H->ndense_];
        return c;
    }();
    StiffDev &S = D.St.S;
    S = StiffDev();
    D.sdofs.upload(sdofs, st);
    D.ssub.upload(ssub, st);
    D.soff.upload(soff, st);
    D.sinvoff.upload(sinvoff, st);
    D.sinv.resize(std::max<int64_t>(inv_at, 1));
    {
        int64_t at = 0;
        for (HybridSolver *H : sys_) {
            if (H->inv_total_ > 0)
                LSS_CUDA(cudaMemcpyAsync(D.sinv.data() + at, H->d_sinv_.data(), (size_t)H->inv_total_ * 8,
                                         cudaMemcpyDeviceToDevice, st));
            at += H->inv_total_;
        }
    }
    D.t.resize(std::max<size_t>(sdofs.size(), 1) * BK);
    S.nsub = nsub;
    S.ndof = (int32_t)sdofs.size();
    S.ndof_dense = ndense_dofs;
    S.dofs = D.sdofs.data();
    S.sub_of = D.ssub.data();
    S.off = D.soff.data();
    S.inv_off = D.sinvoff.data();
    S.inv = D.sinv.data();
    D.St.t = D.t.data();
    // multifrontal: concatenated symbolic structures and front storage
    MfSymbolic MS;
    MS.j_base = ndense_dofs;
    {
        int32_t pos = 0, front = 0, jmf = ndense_dofs;
        int64_t elems = 0;
        int32_t wel = 0, bnd = 0, chi = 0;
        MS.bnd_off.push_back(0);
        MS.child_off.push_back(0);
        MS.foff.push_back(0);
        MS.woff.push_back(0);
        for (int32_t s = 0; s < ns; ++s) {
            const MfSymbolic &Q = sys_[s]->mf_->symbolic();
            const int32_t jm = sys_[s]->h_soff_.back() - sys_[s]->h_soff_[sys_[s]->ndense_];
            if (Q.nfront > 0) {
                // the system's multifrontal DOFs: its j indices from Q.j_base map to merged jmf
                for (int32_t f = 0; f < Q.nfront; ++f) {
                    MS.p0.push_back(Q.p0[f] + pos);
                    MS.s.push_back(Q.s[f]);
                    MS.u.push_back(Q.u[f]);
                    MS.height.push_back(Q.height[f]);
                    MS.foff.push_back(Q.foff[f + 1] + elems);
                    MS.woff.push_back(Q.woff[f + 1] + wel);
                    MS.bnd_off.push_back(Q.bnd_off[f + 1] + bnd);
                    MS.child_off.push_back(Q.child_off[f + 1] + chi);
                    front_sys.push_back(s);
                }
                append(MS.bnd_pos, Q.bnd_pos, pos);
                append(MS.child, Q.child, front);
                append(MS.ea_map, Q.ea_map);
                append(MS.front_of_pos, Q.front_of_pos, front);
                for (int32_t jj : Q.pos2j) MS.pos2j.push_back(jj - Q.j_base + jmf);
                append(MS.j2pos, Q.j2pos, pos);
                MS.levels = std::max(MS.levels, Q.levels);
                MS.max_f = std::max(MS.max_f, Q.max_f);
                MS.max_s = std::max(MS.max_s, Q.max_s);
                MS.fmas += Q.fmas;
                pos += Q.npos;
                front += Q.nfront;
                elems += Q.elems;
                wel += (int32_t)Q.welems;
                bnd += (int32_t)Q.bnd_pos.size();
                chi += (int32_t)Q.child.size();
            }
            jmf += jm;
        }
        MS.nfront = front;
        MS.npos = pos;
        MS.elems = elems;
        MS.welems = wel;
    }
    D.mf = MfFactor();
    if (MS.nfront > 0) {
        D.mf.setup(MS, st);
        int64_t at = 0;
        for (HybridSolver *H : sys_) {
            const MfSymbolic &Q = H->mf_->symbolic();
            if (Q.nfront == 0) continue;
            LSS_CUDA(cudaMemcpyAsync(D.mf.fronts_mut() + at, H->mf_->fronts(), (size_t)Q.elems * 8,
                                     cudaMemcpyDeviceToDevice, st));
            at += Q.elems;
        }
        D.front_sys.upload(front_sys, st);
        D.mf.make_pairs(st);
    }

    // ---- vectors and the device view
    const int64_t nvec = (int64_t)nb * BDIM * BK;
    D.b.resize(nvec);
    D.xt.resize(nvec);
    for (DBuf<float2> *v : {&D.x, &D.r, &D.p, &D.z, &D.ap}) v->resize(nvec);
    D.w.resize(nvec);
    BatchDev &B = D.B;
    B = BatchDev();
    B.nsys = ns;
    B.nb = nb;
    B.nchunk = nchunk;
    B.n = (int64_t)nb * BDIM;
    B.rows = D.rows.data();
    B.cols = D.cols.data();
    B.vals = D.vals.data();
    B.vals32 = D.vals32.data();
    B.vals_df = D.vals_df.data();
    B.precise = any_precise ? D.precise.data() : nullptr;
    B.chunk_sys = D.chunk_sys.data();
    B.chunk_p0 = D.chunk_p0.data();
    B.sys_chunk0 = D.sys_chunk0.data();
    B.part_off = D.part_off.data();
    B.omega = D.omega.data();
    B.lane = D.lane.data();
    B.sys_done = D.sys_done.data();
    B.err = D.sys_done.data() + ns;
    B.partials = D.partials.data();
    B.counters = D.counters.data();
    // scatter table of the user vectors
    LSS_CUDA(cudaStreamSynchronize(st));
    merged_ = true;
}

// ------------------------------------------------------------------ solve

void BatchSolver::precond(int dot_mode)
{
    Impl &D = *d_;
    // z = omega M r (MAS in FP32 on the high words of r)
    bk::launch_mas(D.B, D.M, D.r.data(), nullptr, D.z.data(), false, 0, nullptr, stream_);
    // z += S^T A_SS^-1 S (r - A z)
    bk::launch_stiff(D.B, D.St.S, D.r.data(), D.z.data(), D.St.t, D.z.data(), stream_);
    if (!D.mf.empty()) D.mf.solve_batch(D.St.S, D.St.t, D.z.data(), D.sys_done.data(), D.front_sys.data(), stream_);
    // z += omega M (r - A z), gamma = r.z (beta with dot mode 2)
    bk::launch_residual32(D.B, D.r.data(), D.z.data(), D.w.data(), stream_);
    bk::launch_mas(D.B, D.M, nullptr, D.w.data(), D.z.data(), true, dot_mode, D.r.data(), stream_);
}

void BatchSolver::iteration()
{
    Impl &D = *d_;
    bk::launch_spmm_alpha(D.B, D.p.data(), D.ap.data(), stream_);
    bk::launch_update_xr(D.B, D.x.data(), D.r.data(), D.p.data(), D.ap.data(), stream_);
    precond(2);
    bk::launch_update_p(D.B, D.p.data(), D.z.data(), stream_);
}

void BatchSolver::launch_chunk(int iters)
{
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
        if (cudaGraphGetNodes(g, nullptr, &nodes) == cudaSuccess) graph_nodes_ = nodes;
        launch_count() -= std::min<unsigned long long>(launch_count().load(), nodes);
        LSS_CUDA(cudaGraphInstantiate(&graph_exec_, g, 0));
        cudaGraphDestroy(g);
        graph_iters_ = iters;
    }
    LSS_CUDA(cudaGraphLaunch(graph_exec_, stream_));
    launch_count() += graph_nodes_;
}

void BatchSolver::solve_device(const double *const *d_b, double *const *d_x, int32_t *iterations)
{
    if (!merged_) fail(LSS_ERR_NOT_FACTORIZED, "batched solve before the batched factorize");
    auto t0 = clk::now();
    Impl &D = *d_;
    const int32_t ns = (int32_t)sys_.size();
    const Params &P0 = sys_[0]->p_;
    // user vectors -> [row][BK] in the merged permuted order
    std::vector<bk::ScatterSys> tab(ns);
    std::vector<int64_t> prefix(ns + 1, 0);
    for (int32_t s = 0; s < ns; ++s) {
        tab[s].src = d_b[s];
        tab[s].dst = d_x[s];
        tab[s].nb = D.nb_sys[s];
        tab[s].row0 = D.row0[s];
        tab[s].perm = sys_[s]->d_perm_.data();
        prefix[s + 1] = prefix[s] + (int64_t)D.nb_sys[s] * 3 * BK;
    }
    D.scat.upload(tab, stream_);
    D.scat_prefix.upload(prefix, stream_);
    bk::launch_to_batch(D.scat.data(), ns, D.scat_prefix.data(), prefix[ns], D.b.data(), stream_);
    for (int32_t s = 0; s < ns; ++s) tab[s].src = d_x[s];
    D.scat.upload(tab, stream_);
    bk::launch_to_batch(D.scat.data(), ns, D.scat_prefix.data(), prefix[ns], D.xt.data(), stream_);
    D.x.zero(stream_);
    // lane states
    bk::launch_lane_norms(D.B, D.b.data(), D.rr.data(), stream_);
    D.h_rr.resize((size_t)ns * BK);
    LSS_CUDA(cudaMemcpyAsync(D.h_rr.data(), D.rr.data(), D.h_rr.size() * 8, cudaMemcpyDeviceToHost, stream_));
    LSS_CUDA(cudaStreamSynchronize(stream_));
    D.h_lane.assign((size_t)ns * BK, BatchLane{});
    D.h_done.assign((size_t)ns + 1, 0);  // [ns]: error status
    for (int32_t s = 0; s < ns; ++s) {
        const Params &P = sys_[s]->p_;
        int all = 1;
        for (int k = 0; k < BK; ++k) {
            BatchLane &L = D.h_lane[(size_t)s * BK + k];
            L.bb = D.h_rr[(size_t)s * BK + k];
            if (!std::isfinite(L.bb)) fail(LSS_ERR_NONFINITE, "a right-hand side holds NaN or Inf values");
            L.rel_eps = P.rel_tol * P.rel_tol;
            L.abs_eps = P.abs_tol * P.abs_tol;
            L.max_iter = P.max_iter;
            L.done = !(L.bb > 0.0) ? STOP_CONVERGED_ABS : STOP_RUNNING;  // GPUHybrid.cu:1428-1439: x = 0
            all &= L.done != 0;
        }
        D.h_done[s] = all;
    }
    LSS_CUDA(cudaMemcpyAsync(D.lane.data(), D.h_lane.data(), D.h_lane.size() * sizeof(BatchLane),
                             cudaMemcpyHostToDevice, stream_));
    LSS_CUDA(cudaMemcpyAsync(D.sys_done.data(), D.h_done.data(), (ns + 1) * sizeof(int), cudaMemcpyHostToDevice,
                             stream_));
    D.counters.zero(stream_);
    std::vector<double> target(D.h_lane.size());
    for (size_t q = 0; q < target.size(); ++q) target[q] = D.h_lane[q].rel_eps;
    int launched = 0;
    const int max_iter = [&]() {
        int m = 0;
        for (HybridSolver *H : sys_) m = std::max(m, H->p_.max_iter);
        return m;
    }();
    std::vector<double> prev_res(D.h_lane.size(), INFINITY);
    last_refinements_ = 0;
    for (int attempt = 0;; ++attempt) {
        // r = b - A x (FP64); z = M r; p = z; gamma = r.z; the PCG runs on the
        // correction (x = 0), folded into the FP64 solution after the attempt
        bk::launch_residual64(D.B, D.b.data(), D.xt.data(), D.r.data(), 0, D.rr.data(), stream_);
        precond(1);
        bk::launch_copy_pairs(D.B, D.p.data(), D.z.data(), stream_);
        while (launched < max_iter) {
            const int chunk = std::min(P0.check_every, max_iter - launched);
            launch_chunk(chunk);
            launched += chunk;
            LSS_CUDA(cudaMemcpyAsync(D.h_done.data(), D.sys_done.data(), (ns + 1) * sizeof(int),
                                     cudaMemcpyDeviceToHost, stream_));
            LSS_CUDA(cudaStreamSynchronize(stream_));
            if (D.h_done[ns] != 0)
                fail(LSS_ERR_INTERNAL, "batched MAS: a bulk copy into shared memory did not complete");
            if (std::all_of(D.h_done.begin(), D.h_done.begin() + ns, [](int v) { return v != 0; })) break;
        }
        // true residuals (FP64), per lane
        bk::launch_fold(D.B, D.xt.data(), D.x.data(), stream_);
        bk::launch_residual64(D.B, D.b.data(), D.xt.data(), nullptr, 1, D.rr.data(), stream_);
        LSS_CUDA(cudaMemcpyAsync(D.h_rr.data(), D.rr.data(), D.h_rr.size() * 8, cudaMemcpyDeviceToHost, stream_));
        LSS_CUDA(cudaMemcpyAsync(D.h_lane.data(), D.lane.data(), D.h_lane.size() * sizeof(BatchLane),
                                 cudaMemcpyDeviceToHost, stream_));
        LSS_CUDA(cudaStreamSynchronize(stream_));
        // restart the lanes whose recurrence converged but whose true residual
        // misses the tolerance (as the single-system solve does), while it pays
        bool restart = false;
        for (int32_t s = 0; s < ns; ++s) {
            const int mr = sys_[s]->p_.max_refinements;
            int all = 1;
            for (int k = 0; k < BK; ++k) {
                const size_t q = (size_t)s * BK + k;
                BatchLane &L = D.h_lane[q];
                const double res2 = D.h_rr[q];
                const bool conv = L.done == STOP_CONVERGED_REL || L.done == STOP_CONVERGED_ABS;
                const bool ok = !(target[q] > 0) || !(L.bb > 0) || res2 / L.bb <= 0.9604 * target[q];
                const bool improving = res2 < 0.25 * prev_res[q];
                prev_res[q] = res2;
                if (conv && L.bb > 0 && !ok && improving && attempt < mr && launched < max_iter) {
                    const double true_rel = std::sqrt(res2 / L.bb);
                    const double tol = std::sqrt(target[q]);
                    const double tgt = tol * std::min(1.0, 0.5 * tol / true_rel);
                    L.rel_eps = tgt * tgt;
                    L.done = STOP_RUNNING;
                    restart = true;
                }
                all &= L.done != 0;
            }
            D.h_done[s] = all;
        }
        if (!restart) break;
        ++last_refinements_;
        LSS_CUDA(cudaMemcpyAsync(D.lane.data(), D.h_lane.data(), D.h_lane.size() * sizeof(BatchLane),
                                 cudaMemcpyHostToDevice, stream_));
        LSS_CUDA(cudaMemcpyAsync(D.sys_done.data(), D.h_done.data(), ns * sizeof(int), cudaMemcpyHostToDevice,
                                 stream_));
    }
    // x -> user vectors (x = 0 where b = 0)
    bk::launch_zero_done_lanes(D.B, D.xt.data(), stream_);
    for (int32_t s = 0; s < ns; ++s) tab[s].dst = d_x[s];
    D.scat.upload(tab, stream_);
    bk::launch_from_batch(D.scat.data(), ns, D.scat_prefix.data(), prefix[ns], D.xt.data(), stream_);
    LSS_CUDA(cudaStreamSynchronize(stream_));
    last_iters_.assign((size_t)ns * BK, 0);
    for (size_t q = 0; q < last_iters_.size(); ++q) last_iters_[q] = D.h_lane[q].iter;
    if (iterations) std::copy(last_iters_.begin(), last_iters_.end(), iterations);
    last_solve_s_ = secs(t0);
}

std::string BatchSolver::info_json() const
{
    std::ostringstream o;
    o.precision(17);
    int mx = 0;
    double mean = 0.0;
    for (int v : last_iters_) {
        mx = std::max(mx, v);
        mean += v;
    }
    if (!last_iters_.empty()) mean /= (double)last_iters_.size();
    o << "{\"systems\": " << sys_.size() << ", \"rhs_per_system\": " << BK << ", \"max_iterations\": " << mx
      << ", \"mean_iterations\": " << mean << ", \"refinements\": " << last_refinements_
      << ", \"time_factorize\": " << last_factorize_s_ << ", \"time_merge\": " << last_merge_s_
      << ", \"time_solve\": " << last_solve_s_ << ", \"kernels_per_chunk\": " << graph_nodes_
      << ", \"kernel_launches\": " << launch_count().load() << ", \"chunks\": " << d_->B.nchunk
      << ", \"mas_levels\": " << d_->M.m.L << ", \"multifrontal_fronts\": " << d_->mf.symbolic().nfront << "}";
    return o.str();
}

}  // namespace lss
