// Pattern analysis: block graph, partition, permuted row-sliced BSR layout
// with its value map, and the MAS coarse space.  Pattern-only, so it is built
// once (analyze_pattern) and reused by every factorize with the same pattern.
#pragma once

#include <cstdint>
#include <vector>

#include "partition.hpp"

namespace lss {

struct Pattern {
    int32_t n = 0, bd = 1, nb = 0;
    int64_t nnz = 0;
    uint64_t hash = 0;                 // of outer/inner, to detect a new pattern
    Partition part;                    // perm (old block -> new), part_offsets
    std::vector<int32_t> iperm;        // new block -> old
    std::vector<int32_t> rows, cols;   // permuted BSR (nb+1, nnzb), cols ascending per row
    std::vector<int64_t> src;          // nnzb*bd*bd: BSR slot -> input entry index, -1 = structural zero
    double mean_blocks_per_row = 0;
};

uint64_t pattern_hash(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner);

// Throws lss::Error on invalid input (indices out of range, duplicates, n % bd).
Pattern analyze_pattern(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner, int bd, int threads);

// MAS coarse space (MASPreconditioner.cu:376-481 semantics) on the permuted
// block graph: level 0 = partitions, level l >= 1 = bank-local connected
// components of level l-1 grouped 32 per bank.
struct CoarseSpace {
    int L = 1;                                    // matrix levels incl. level 0
    std::vector<int32_t> part_of;                 // nb
    std::vector<uint8_t> key0;                    // nb
    std::vector<int32_t> cbase0;                  // nparts
    std::vector<uint8_t> ccnt0;                   // nparts
    std::vector<int32_t> nitems, nbanks;          // per level (level 0: nodes / parts)
    std::vector<std::vector<uint8_t>> key;        // level l: nbanks[l]*32 (padded)
    std::vector<std::vector<int32_t>> cbase;      // level l: nbanks[l]
    std::vector<std::vector<uint8_t>> ccnt;       // level l: nbanks[l]
    std::vector<int32_t> cmap;                    // (L-1) * nb: item of every node at level l
    // members of every coarse item, levels 1..L-1 concatenated: item t of level
    // l owns memb_rows[memb_ptr[memb_base[l] + t] .. memb_ptr[memb_base[l] + t + 1])
    // (fine block rows, ascending) -- the fixed summation order of the
    // deterministic Galerkin assembly
    std::vector<int32_t> memb_ptr, memb_rows;
    std::vector<int64_t> memb_base;               // L entries (level 0 unused)
    // the members split into chunks of at most MEMB_CHUNK rows (one warp
    // each); item i (flat over levels 1..L-1) owns chunks
    // [item_chunk[i], item_chunk[i+1]); chunk c covers memb_rows[chunk_r0[c] ..
    // chunk_r0[c+1]) -- consecutive chunks of an item are contiguous
    std::vector<int32_t> item_chunk, chunk_r0;
};
constexpr int32_t MEMB_CHUNK = 128;

CoarseSpace build_coarse_space(const Pattern &P, int max_coarse_levels);

}  // namespace lss
