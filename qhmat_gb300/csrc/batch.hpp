// Block-diagonal concatenation of independent matrices (the batching form).
#pragma once

#include <cstdint>
#include <vector>

#include "layout.hpp"

namespace qhg {

// diag(ms[0], ms[1], ...): matrix k occupies rows and columns [offsets[k],
// offsets[k] + ms[k].order), each offset a multiple of `align`; rows between
// matrices belong to no block.
HostMatrix concat_block_diagonal(const std::vector<HostMatrix>& ms, uint64_t align, std::vector<uint64_t>& offsets);

}  // namespace qhg
