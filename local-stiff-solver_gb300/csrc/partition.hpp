// Partition of the block graph into parts of <= 32 block rows (MAS banks).
#pragma once

#include <cstdint>
#include <vector>

namespace lss {

struct Partition {
    std::vector<int32_t> perm;          // old block row -> new block row
    std::vector<int32_t> part_offsets;  // nparts + 1, in the new numbering
};

// rows/cols: symmetric block graph without self loops.
Partition partition_graph(int32_t nb, const int32_t *rows, const int32_t *cols, int threads);

}  // namespace lss
