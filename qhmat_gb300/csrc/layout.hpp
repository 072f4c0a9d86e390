// Host-side ingestion of a quantized H-matrix and the resident device layout.
//
// The layout is built once per matrix on the host and uploaded as a single
// arena; every kernel reads only this arena plus the caller's x, y and
// workspace.  Nothing here depends on CUDA, so the builder is unit-testable
// on the CPU.
//
// Code words keep the reference's bit packing (component j of width w_j,
// LSB-first, code i at bit i*w_j of the component's run) but the 32-bit words
// are permuted so that each kernel reads them coalesced:
//
//  * right factor Q (column side): components are grouped into tasks of at
//    most 32 components that share a column range and a width; lane l of a
//    warp owns component l of its task.  For chunk c (entries 32c..32c+31)
//    the chunk's w words of lane l's run sit at
//        qwords[task.word0 + c*w*count + v*count + l],  v = 0..w-1,
//    so a warp loading word v of its chunk reads `count` consecutive words.
//  * left factor P (row side): rows are cut into tiles of at most 64 rows
//    inside one elementary row slab.  For each (tile, block covering it) the
//    pieces of the block's components for the tile's rows are stored back to
//    back: component j's piece is the bit string [r0*w_j, (r0+rows)*w_j) of
//    its run (r0 = tile row - block row0), starting at a fresh word and
//    occupying ceil(rows*w_j/32) words.
//  * dense diagonal blocks are stored column-major (value (i, k) at
//    off + k*m + i) so that lanes owning consecutive rows read consecutive
//    doubles.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace qhg {

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
        uint64_t dense_off = 0;   // dense only: offset into `dense` (row-major)
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

// Rows of one row tile at most (one CTA of the row-side kernel).
constexpr int kTileRows = 64;
// Entries of one column-side chunk (one code per lane per entry).
constexpr int kColChunk = 32;
// x entries per exponent chunk of the fixed-point right-hand side.
constexpr int kChunk = 32;

// QHMAT001 trailer: FNV-1a-64 (src/qhmat/io.cpp:18-19).
constexpr uint64_t kFnvOffsetBasis = 14695981039346656037ULL;
constexpr uint64_t kFnvPrimeValue = 1099511628211ULL;

// Device-side descriptors (32-bit indices; checked by build_layout).
struct LowRankDesc {
    int32_t row0, m, col0, n;
    int32_t rank, comp0;
};
// Column-side unit of work: chunks [chunk0, chunk0 + nchunks) of a task of
// `count` (<= 32) components of width `width` whose blocks share the column
// range [col0, col0 + n).  Chunk c of the task starts at word
// word0 + c * stride (16-byte aligned; stride = `count * width` rounded up to
// a multiple of 4 words) and holds word v of lane l at + v * count + l.
// A task longer than kMaxPartChunks chunks is split into `nparts` parts whose
// partial sums are combined by the part that finishes last.
struct ColTask {
    int32_t col0, n, width, count;
    int64_t word0;
    int32_t stride, comp_idx;   // comp_idx: first of `count` entries in task_comp
    int32_t chunk0, nchunks;
    int32_t part, nparts;
    int32_t split_id;           // index of the split task (counter / partials), -1 if nparts == 1
    int32_t pad;
};
// Row-side unit of work: components [j0, j0 + count) of one low-rank block for
// one row tile, or a column slice of one dense block for one row tile (dense:
// comp = slice index, count = columns, words = first column, off = element
// offset of (first row, first column) in the column-major values).  Low-rank
// data block at pwords[off]: kRowHeaderWords header words holding, for each
// of the `count` components, a 16-bit entry (piece offset in words << 5) |
// (width - 1); then the pieces (component j's piece = bits [rloc0*w,
// (rloc0 + rows)*w) of its run, from a fresh word, ceil(rows*w/32) words);
// `words` is the block's total size, a multiple of 4 words, 16-byte aligned.
struct RowItem {
    int32_t block;     // >= 0: low-rank block index; < 0: -1 - dense block index
    int32_t rloc0;     // tile row0 - block row0
    int32_t comp, count;  // first component id (block comp0 + j0), components in the unit
    int64_t off;       // low-rank: word offset of the data block; dense: element offset
    int32_t words, pad;
};
struct DenseDesc {
    int32_t row0, m, col0, n;
    int64_t off;  // element offset of the column-major values in the dense arena
};
struct RowTile {
    int32_t row0, rows;     // clustered rows [row0, row0+rows), inside one slab
    int32_t item0, item1;   // range in the items array (the tile's units)
};

// Shared-memory stage of one warp's prefetch pipeline (bytes of code words).
constexpr int kStageWordBytes = 4096;
// Longest run of chunks one column unit walks.
constexpr int kMaxPartChunks = 16;
// Header words of a row data block (32 16-bit offset/width entries).
constexpr int kRowHeaderWords = 16;
// Column slices a dense diagonal block is cut into (one per row-side warp).
constexpr int kDenseSlices = 8;

// Byte offsets of each section inside the device arena.
struct Sections {
    size_t perm, lr, dd, comp_w, comp_s, tasks, task_comp, qwords, pwords, dense, tiles, items;
    size_t total;
};

struct Layout {
    uint64_t order = 0;
    int32_t n_lr = 0, n_dense = 0, n_comp = 0, n_tiles = 0, n_items = 0, n_chunks = 0;
    int32_t n_tasks = 0, n_split = 0, max_parts = 1;
    std::vector<uint8_t> arena;  // host image of the device arena
    Sections sec{};
    double bound = 0;
    // traffic model (reference word counts) and stored sizes
    uint64_t code_bytes = 0, left_code_bytes = 0, right_code_bytes = 0, scale_bytes = 0,
             dense_bytes = 0, flops = 0;
    uint64_t stored_q_words = 0, stored_p_words = 0;
};

Layout build_layout(const HostMatrix& m);

// Words of the bit string of `rows` codes of width w.
inline uint64_t words_for_bits(uint64_t rows, int w) { return (rows * uint64_t(w) + 31) / 32; }

}  // namespace qhg
