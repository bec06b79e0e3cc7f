// Pattern analysis and MAS coarse space construction (host, threaded).
//
// Block graph + partition replace BSRAdjacency + GraphPartition
// (BSRAdjacency.cu:164-493, GraphPartition.cpp:176-289); the permuted BSR
// replaces BSRMatrix (BSRMatrix.cu:195-474) with the row-sliced value layout
// of spmv.cuh and a gather map, so refactorising with new values is a single
// device gather.  The coarse space restates build_coarse_space
// (MASPreconditioner.cu:128-481): components inside each bank found by
// bit-mask closure, numbered per bank by lowest lane, globally by bank order.
#include <algorithm>
#include <thread>

#include "lss_common.hpp"
#include "pattern.hpp"

namespace lss {
namespace {

template <typename F>
void parallel_for(int64_t n, int threads, F f)
{
    if (threads <= 1 || n < 4096) {
        f(0, n, 0);
        return;
    }
    std::vector<std::thread> th;
    const int64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([=, &f]() { f(lo, hi, t); });
    }
    for (auto &x : th) x.join();
}

int default_threads(int t)
{
    if (t > 0) return t;
    return (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
}

}  // namespace

uint64_t pattern_hash(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner)
{
    // FNV-1a over a strided sample plus the full outer array
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](uint64_t v) {
        h ^= v;
        h *= 1099511628211ull;
    };
    mix((uint64_t)n);
    mix((uint64_t)nnz);
    for (int32_t i = 0; i <= n; ++i) mix((uint64_t)(uint32_t)outer[i]);
    const int64_t step = std::max<int64_t>(1, nnz / 1000003);
    for (int64_t k = 0; k < nnz; k += step) mix((uint64_t)(uint32_t)inner[k] ^ ((uint64_t)k << 32));
    return h;
}

Pattern analyze_pattern(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner, int bd, int threads)
{
    threads = default_threads(threads);
    if (n <= 0) fail(LSS_ERR_INVALID_ARGUMENT, "matrix dimension must be positive");
    if (n % bd != 0)
        fail(LSS_ERR_INVALID_ARGUMENT, "matrix dimension " + std::to_string(n) + " is not a multiple of block_size " +
                                           std::to_string(bd));
    if (outer[0] != 0 || (int64_t)outer[n] != nnz)
        fail(LSS_ERR_INVALID_ARGUMENT, "outer index must start at 0 and end at nnz (compressed storage)");
    for (int32_t i = 0; i < n; ++i)
        if (outer[i + 1] < outer[i]) fail(LSS_ERR_INVALID_ARGUMENT, "outer index is not monotone");
    Pattern P;
    P.n = n;
    P.bd = bd;
    P.nb = n / bd;
    P.nnz = nnz;
    P.hash = pattern_hash(n, nnz, outer, inner);
    const int32_t nb = P.nb;

    // ---- block graph in the input numbering (no self loops)
    std::vector<int32_t> cnt(nb + 1, 0);
    std::vector<int> bad(threads, 0);
    parallel_for(nb, threads, [&](int64_t lo, int64_t hi, int t) {
        std::vector<int32_t> mark(nb, -1);
        for (int64_t o = lo; o < hi; ++o) {
            int32_t c = 0;
            for (int r = 0; r < bd; ++r)
                for (int32_t k = outer[o * bd + r]; k < outer[o * bd + r + 1]; ++k) {
                    const int32_t col = inner[k];
                    if (col < 0 || col >= n) { bad[t] = 1; continue; }
                    const int32_t J = col / bd;
                    if (mark[J] != (int32_t)o) { mark[J] = (int32_t)o; ++c; }
                }
            cnt[o + 1] = c;  // blocks of the row incl. the diagonal block
        }
    });
    for (int b : bad)
        if (b) fail(LSS_ERR_INVALID_ARGUMENT, "inner index out of range");
    std::vector<int32_t> brow(nb + 1, 0);
    for (int32_t o = 0; o < nb; ++o) brow[o + 1] = brow[o] + cnt[o + 1];
    std::vector<int32_t> bcol(brow[nb]);
    std::vector<int32_t> grow(nb + 1, 0);
    parallel_for(nb, threads, [&](int64_t lo, int64_t hi, int) {
        std::vector<int32_t> mark(nb, -1);
        for (int64_t o = lo; o < hi; ++o) {
            int32_t pos = brow[o];
            for (int r = 0; r < bd; ++r)
                for (int32_t k = outer[o * bd + r]; k < outer[o * bd + r + 1]; ++k) {
                    const int32_t J = inner[k] / bd;
                    if (mark[J] != (int32_t)o) { mark[J] = (int32_t)o; bcol[pos++] = J; }
                }
            std::sort(bcol.begin() + brow[o], bcol.begin() + brow[o + 1]);
            int32_t self = 0;
            for (int32_t k = brow[o]; k < brow[o + 1]; ++k) self += bcol[k] == (int32_t)o;
            grow[o + 1] = brow[o + 1] - brow[o] - self;
        }
    });
    for (int32_t o = 0; o < nb; ++o) grow[o + 1] += grow[o];
    std::vector<int32_t> gcol(grow[nb]);
    parallel_for(nb, threads, [&](int64_t lo, int64_t hi, int) {
        for (int64_t o = lo; o < hi; ++o) {
            int32_t pos = grow[o];
            for (int32_t k = brow[o]; k < brow[o + 1]; ++k)
                if (bcol[k] != (int32_t)o) gcol[pos++] = bcol[k];
        }
    });

    // ---- partition
    P.part = partition_graph(nb, grow.data(), gcol.data(), threads);
    P.iperm.assign(nb, -1);
    for (int32_t o = 0; o < nb; ++o) P.iperm[P.part.perm[o]] = o;

    // ---- permuted BSR pattern + value map
    P.rows.assign(nb + 1, 0);
    for (int32_t I = 0; I < nb; ++I) {
        const int32_t o = P.iperm[I];
        P.rows[I + 1] = P.rows[I] + (brow[o + 1] - brow[o]);
    }
    const int64_t nnzb = P.rows[nb];
    const int bd2 = bd * bd;
    if (nnzb * bd2 > (int64_t)0x7fffffff * 4) fail(LSS_ERR_UNSUPPORTED, "matrix too large: more than 2^33 block values");
    P.cols.assign(nnzb, 0);
    P.src.assign(nnzb * bd2, -1);
    std::vector<int> dup(threads, 0);
    parallel_for(nb, threads, [&](int64_t lo, int64_t hi, int t) {
        std::vector<int32_t> slot(nb, -1);
        for (int64_t I = lo; I < hi; ++I) {
            const int32_t o = P.iperm[I];
            const int32_t b = P.rows[I], len = P.rows[I + 1] - b;
            for (int32_t q = 0; q < len; ++q) P.cols[b + q] = P.part.perm[bcol[brow[o] + q]];
            std::sort(P.cols.begin() + b, P.cols.begin() + b + len);
            for (int32_t q = 0; q < len; ++q) slot[P.cols[b + q]] = q;
            for (int r = 0; r < bd; ++r)
                for (int32_t k = outer[o * bd + r]; k < outer[o * bd + r + 1]; ++k) {
                    const int32_t col = inner[k];
                    const int32_t q = slot[P.part.perm[col / bd]];
                    const int64_t idx = (int64_t)b * bd2 + (int64_t)(r * bd + col % bd) * len + q;
                    if (P.src[idx] != -1) dup[t] = 1;
                    P.src[idx] = k;
                }
            for (int32_t q = 0; q < len; ++q) slot[P.cols[b + q]] = -1;
        }
    });
    for (int d : dup)
        if (d) fail(LSS_ERR_INVALID_ARGUMENT, "duplicate entries in the compressed matrix");
    P.mean_blocks_per_row = nb ? (double)nnzb / nb : 0.0;
    return P;
}

namespace {

// bank-local components: items 0..nitems-1 in banks of 32, masks[item] holds
// in-bank neighbour bits incl. self.  Writes local ids, per-bank counts.
void bank_components(int32_t nitems, const std::vector<uint32_t> &masks, std::vector<uint8_t> &key,
                     std::vector<uint8_t> &ccnt, std::vector<int32_t> &cbase, int32_t &total,
                     const std::vector<char> *valid = nullptr)
{
    const int32_t nbank = (nitems + 31) / 32;
    key.assign((size_t)nbank * 32, 0);
    ccnt.assign(nbank, 0);
    cbase.assign(nbank, 0);
    total = 0;
    for (int32_t b = 0; b < nbank; ++b) {
        int lead[32];
        uint32_t leads = 0;
        for (int l = 0; l < 32; ++l) {
            const int32_t t = b * 32 + l;
            lead[l] = -1;
            if (t >= nitems || (valid && !(*valid)[t])) continue;
            uint32_t conn = masks[t], visited = 1u << l, to_visit = conn ^ visited;
            while (to_visit) {
                const int v = __builtin_ctz(to_visit);
                conn |= masks[b * 32 + v];
                visited |= 1u << v;
                to_visit = conn ^ visited;
            }
            lead[l] = __builtin_ctz(conn);
            if (lead[l] == l) leads |= 1u << l;
        }
        for (int l = 0; l < 32; ++l) {
            const int32_t t = b * 32 + l;
            if (lead[l] < 0) continue;
            const uint32_t before = (uint32_t)((1ull << lead[l]) - 1ull);
            key[t] = (uint8_t)__builtin_popcount(leads & before);
        }
        ccnt[b] = (uint8_t)__builtin_popcount(leads);
        cbase[b] = total;
        total += __builtin_popcount(leads);
    }
}

}  // namespace

CoarseSpace build_coarse_space(const Pattern &P, int max_coarse_levels)
{
    CoarseSpace cs;
    const int32_t nb = P.nb;
    const auto &po = P.part.part_offsets;
    const int32_t nparts = (int32_t)po.size() - 1;
    cs.part_of.assign(nb, 0);
    for (int32_t p = 0; p < nparts; ++p)
        for (int32_t i = po[p]; i < po[p + 1]; ++i) cs.part_of[i] = p;

    // level 0 components inside each partition (padded banks of 32 lanes)
    {
        std::vector<uint32_t> masks((size_t)nparts * 32, 0);
        std::vector<char> valid((size_t)nparts * 32, 0);
        for (int32_t i = 0; i < nb; ++i) {
            const int32_t p = cs.part_of[i], lane = i - po[p];
            const int64_t t = (int64_t)p * 32 + lane;
            valid[t] = 1;
            uint32_t m = 1u << lane;
            for (int32_t k = P.rows[i]; k < P.rows[i + 1]; ++k) {
                const int32_t j = P.cols[k];
                if (j >= po[p] && j < po[p + 1]) m |= 1u << (j - po[p]);
            }
            masks[t] = m;
        }
        std::vector<uint8_t> key;
        int32_t total = 0;
        bank_components(nparts * 32, masks, key, cs.ccnt0, cs.cbase0, total, &valid);
        cs.key0.assign(nb, 0);
        for (int32_t i = 0; i < nb; ++i) cs.key0[i] = key[(int64_t)cs.part_of[i] * 32 + (i - po[cs.part_of[i]])];
        cs.nitems = {nb, total};
        cs.nbanks = {nparts, (total + 31) / 32};
        cs.cmap.resize(nb);
        for (int32_t i = 0; i < nb; ++i) cs.cmap[i] = cs.cbase0[cs.part_of[i]] + cs.key0[i];
    }
    cs.key.resize(2);
    cs.cbase.resize(2);
    cs.ccnt.resize(2);
    int L = 2;
    // coarser levels (MASPreconditioner.cu:424-474)
    for (int l = 1; l < max_coarse_levels; ++l) {
        const int32_t items = cs.nitems[l];
        const int32_t *map = cs.cmap.data() + (int64_t)(l - 1) * nb;
        std::vector<uint32_t> masks(((size_t)items + 31) / 32 * 32, 0);
        for (int32_t t = 0; t < items; ++t) masks[t] = 1u << (t & 31);
        for (int32_t i = 0; i < nb; ++i) {
            const int32_t a = map[i];
            for (int32_t k = P.rows[i]; k < P.rows[i + 1]; ++k) {
                const int32_t b = map[P.cols[k]];
                if (a != b && (a >> 5) == (b >> 5)) {
                    masks[a] |= 1u << (b & 31);
                    masks[b] |= 1u << (a & 31);
                }
            }
        }
        std::vector<uint8_t> key, ccnt;
        std::vector<int32_t> cbase;
        int32_t next = 0;
        bank_components(items, masks, key, ccnt, cbase, next);
        if (next == items) break;  // no more components to merge
        cs.key[l] = std::move(key);
        cs.ccnt[l] = std::move(ccnt);
        cs.cbase[l] = std::move(cbase);
        cs.cmap.resize((size_t)l * nb + nb);
        int32_t *nmap = cs.cmap.data() + (int64_t)l * nb;
        const int32_t *pmap = cs.cmap.data() + (int64_t)(l - 1) * nb;
        for (int32_t i = 0; i < nb; ++i) {
            const int32_t a = pmap[i];
            nmap[i] = cs.cbase[l][a >> 5] + cs.key[l][a];
        }
        cs.nitems.push_back(next);
        cs.nbanks.push_back((next + 31) / 32);
        L = l + 2;
        cs.key.resize(L);
        cs.cbase.resize(L);
        cs.ccnt.resize(L);
    }
    cs.L = L;
    cs.key.resize(L);
    cs.cbase.resize(L);
    cs.ccnt.resize(L);
    // member lists (counting sort of cmap per level; rows ascending)
    cs.memb_base.assign(L, 0);
    cs.memb_rows.resize((size_t)(L - 1) * nb);
    for (int l = 1; l < L; ++l) {
        const int32_t items = cs.nitems[l];
        const int32_t *map = cs.cmap.data() + (int64_t)(l - 1) * nb;
        const int64_t base = (int64_t)cs.memb_ptr.size();
        cs.memb_base[l] = base;
        cs.memb_ptr.resize(base + items + 1, 0);
        int32_t *ptr = cs.memb_ptr.data() + base;
        for (int32_t i = 0; i < nb; ++i) ++ptr[map[i] + 1];
        const int32_t first = (int32_t)((int64_t)(l - 1) * nb);
        ptr[0] = first;
        for (int32_t t = 0; t < items; ++t) ptr[t + 1] += ptr[t];
        std::vector<int32_t> fill(ptr, ptr + items);
        for (int32_t i = 0; i < nb; ++i) cs.memb_rows[fill[map[i]]++] = i;
    }
    cs.item_chunk.assign(1, 0);
    for (int l = 1; l < L; ++l) {
        const int32_t *ptr = cs.memb_ptr.data() + cs.memb_base[l];
        for (int32_t t = 0; t < cs.nitems[l]; ++t) {
            for (int32_t r = ptr[t]; r < ptr[t + 1]; r += MEMB_CHUNK) cs.chunk_r0.push_back(r);
            cs.item_chunk.push_back((int32_t)cs.chunk_r0.size());
        }
    }
    cs.chunk_r0.push_back((int32_t)cs.memb_rows.size());  // end of the last chunk
    return cs;
}

}  // namespace lss
