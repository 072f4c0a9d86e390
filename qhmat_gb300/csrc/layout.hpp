// Host-side ingestion of a quantized H-matrix and the resident device layout.
//
// The layout is built once per matrix on the host and uploaded as a single
// arena; every kernel reads only this arena plus the caller's x, y and
// workspace.  Nothing here depends on CUDA, so the builder is unit-testable
// on the CPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace qhg {

// Exceptions carry the reference's exception class, mapped to QH_* codes at
// the C ABI: invalid_argument -> QH_EINVAL, runtime_error -> QH_ERUNTIME,
// overflow_error -> QH_EOVERFLOW.
using std::invalid_argument;
using std::overflow_error;
using std::runtime_error;

// Flattened host copy of a matrix, in the reference's block insertion order.
struct HostMatrix {
    uint64_t order = 0;
    std::vector<uint64_t> permutation;  // clustered position -> source index

    struct Block {
        uint64_t row0, row1, col0, col1;
        bool admissible, dense;
        uint64_t rank = 0;        // low-rank only
        uint64_t comp0 = 0;       // first component index
        uint64_t dense_off = 0;   // dense only: offset into `dense`
        double truncation_error = 0, quantization_bound = 0;
    };
    std::vector<Block> blocks;

    // Per component (low-rank blocks, concatenated in block order).
    std::vector<uint8_t> width;
    std::vector<double> left_scale, right_scale;
    std::vector<uint64_t> left_off, right_off;  // word index into left_words/right_words
    std::vector<uint32_t> left_words, right_words;
    std::vector<double> dense;

    double reconstruction_bound() const;
};

// QHMAT001 image -> HostMatrix, with the checks and messages of
// HMatrix::load (io.cpp:173-257), the permutation check of the HMatrix
// constructor (core.cpp:205-212), check_rectangle (core.cpp:214-222) and
// finalize (core.cpp:332-358).
HostMatrix parse_qhmat(const uint8_t* bytes, size_t len);

// Validate a HostMatrix assembled from caller arrays (permutation bijection,
// rectangles, ranks, widths, finite values, partition cover).
void validate(const HostMatrix& m);

// Device-side descriptors.  All indices are 32-bit: one matrix holds fewer
// than 2^31 rows, blocks and components and fewer than 2^32 code words per
// factor side (checked by build_layout).
struct LowRankDesc {
    int32_t row0, m, col0, n;
    int32_t rank, comp0;
};
struct DenseDesc {
    int32_t row0, m, col0, n;
    int64_t off;  // element offset into the dense arena
};
struct RowTile {
    int32_t row0, rows;     // clustered rows [row0, row0+rows), inside one slab
    int32_t item0, item1;   // range in the items array (the slab's blocks)
};

// Byte offsets of each section inside the device arena.
struct Sections {
    size_t perm, lr, dd, comp_w, comp_s, comp_qoff, comp_poff, qwords, pwords, dense;
    size_t a_order, tiles, items;
    size_t total;
};

struct Layout {
    uint64_t order = 0;
    int32_t n_lr = 0, n_dense = 0, n_comp = 0, n_tiles = 0, n_items = 0, n_chunks = 0;
    int32_t n_a = 0;                  // low-rank blocks with rank > 0 (column-side work)
    int32_t max_tile_items_comp = 0;  // largest sum of ranks over one tile's items
    std::vector<uint8_t> arena;       // host image of the device arena
    Sections sec{};
    double bound = 0;
    // traffic model
    uint64_t code_bytes = 0, scale_bytes = 0, dense_bytes = 0, flops = 0;
};

Layout build_layout(const HostMatrix& m);

// QHMAT001 trailer: FNV-1a-64 (src/qhmat/io.cpp:18-19).
constexpr uint64_t kFnvOffsetBasis = 14695981039346656037ULL;
constexpr uint64_t kFnvPrimeValue = 1099511628211ULL;

// Rows of one row tile at most (one CTA of the row-side kernel).
constexpr int kTileRows = 64;
// x entries per exponent chunk of the fixed-point right-hand side.
constexpr int kChunk = 32;

}  // namespace qhg
