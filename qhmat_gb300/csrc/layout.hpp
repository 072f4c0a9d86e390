// Host-side ingestion of a quantized H-matrix and the resident device layout.
//
// The layout is built once per matrix on the host and uploaded as a single
// arena; every kernel reads only this arena plus the caller's x, y and
// workspace.  Nothing here depends on CUDA, so the builder is unit-testable
// on the CPU.
//
// Codes are stored as digit planes laid out for the tensor cores.  A code c of
// width w (two's complement) on P = ceil(w/8) planes with t = w - 8(P-1) top
// bits is
//     c = sum_{m<P-1} 2^(8m) d_m + 2^(8(P-1)) (d_top - 2^(t-1)),
// d_m = (c >> 8m) & 255 and d_top = (c >> 8(P-1)) + 2^(t-1) in [0, 2^t)
// (stored as a nibble when t <= 4).  The device reads the top digit as the
// signed d_top - 2^(t-1), so
//     sum_i c_i v_i = sum_m 2^(8m) sum_i digit_m,i v_i
// with no offset correction, and every inner sum is an exact small-integer
// product sum (|digits| <= 255 times 8-bit limbs of the fixed-point operand),
// which the f16 tensor-core MMA computes exactly in FP32 (no partial sum
// reaches 2^24).  Digits are
// grouped into the 16x16 A-operand fragments of mma.m16n8k16: within a
// 16-entry k-block, thread t of a fragment row needs entries 2t, 2t+1, 2t+8,
// 2t+9, and those four digits are stored together:
//   byte group row (32 bytes per 2 k-blocks): bytes 8t..8t+3 = k-block 0
//     entries (2t, 2t+1, 2t+8, 2t+9), bytes 8t+4..8t+7 = k-block 1;
//   nibble group row (16 bytes per 2 k-blocks): word t, nibble k (k = 0..3:
//     k-block k>>1, entry 2t + 8(k&1)) and nibble k+4 (the following entry).
//
//  * right factor Q (column side): components sharing a column range and a
//    width form tasks of <= 32 (two 16-row M-tiles).  Per 32-entry chunk a
//    task stores, for each M-tile q and plane m, the group of its rows_q rows;
//    entries past the range hold code 0.
//  * left factor P (row side): rows are cut into tiles of <= 64 rows inside
//    one elementary row slab.  The components of all blocks covering a tile
//    are sorted by width, widest first, and form the tile's k axis (k-pairs
//    of 32).  A k-pair's codes are all written on the planes of its widest
//    code (P and t of that width; narrower codes sign-extended).  The tile's
//    M-tile q (16 rows) and k split h own one contiguous stream (a row unit):
//    for every k-pair kp = h, h + H, ... and every plane m of the k-pair, one
//    group of 16 rows (zero past the tile or past the k axis).  Each k slot
//    has a B row, written for every apply by the column task that computes
//    its component: the eight f16 limbs of U = u in fixed point on the tile's
//    exponent; a unit's B rows are contiguous (slot = tile base + h's base +
//    32 i + lane for its i-th k-pair).
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

// Rows of one row tile at most.
constexpr int kTileRows = 64;
// Row units of one tile at most: its M-tiles (16 rows each) times the k
// splits, hsplit = kTileUnits / M-tiles.
constexpr int kTileUnits = 8;
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
// range [col0, col0 + n).  Chunk c of the task starts at byte off + c * stride
// and holds, for M-tile q (rows_q = min(16, count - 16q)) and plane m, rows_q
// rows of 32 bytes (16 for a nibble top plane).  A pipeline step carries
// `cps` chunks.  A task longer than kMaxPartChunks chunks is split into
// `nparts` parts whose partial sums are combined by the part that finishes
// last.  The task's components feed ndest row-side B rows, listed at
// task_dest[dest0 ..] (every part holds the same list; the finishing part
// writes them).  A unit of width 0 instead holds columns [chunk0, chunk0 + n)
// of the dense diagonal block part tdense[col0] of row tile `stride`, its row
// sums going to dense slice comp_idx.
struct ColTask {
    int32_t col0, n, count, width;
    int64_t off;
    int32_t stride, comp_idx;   // comp_idx: first of `count` entries in task_rec
    int32_t chunk0, nchunks;
    int32_t part, nparts;
    int32_t split_id;           // index of the split task (counter / partials), -1 if nparts == 1
    int32_t cps;
    int32_t dest0, ndest;
};
// A row-side B row fed by a column task: slot, and (component row in the
// task) << 16 | the tile's exponent offset as a 16-bit signed field.  A task's
// list is ordered by (tile, row), so that a tile's B rows are consecutive.
struct TaskDest {
    int32_t slot, row_cexp;
};
static_assert(sizeof(TaskDest) == 8, "TaskDest layout");
static_assert(sizeof(ColTask) == 64, "ColTask layout");
// Finalize operands of one component of a column task (one 16-byte load).
struct TaskRec {
    int32_t comp, width;
    double scale;  // s^P s^Q
};
struct DenseDesc {
    int32_t row0, m, col0, n;
    int64_t off;  // element offset of the column-major values in the dense arena
};
// One row tile: clustered rows [row0, row0 + rows) inside one slab; qrows
// M-tiles, k axis split hsplit ways (nh of the splits have k-pairs); dense
// blocks tdense[dense0 .. dense0 + ndense), whose row sums are kept as dense
// slices ds0 .. ds0 + nds - 1 (kDenseCols columns each, in column order); u
// is put in fixed point on the exponent field xe + c_exp (xe: the largest
// exponent field of x).
struct RowTile {
    int32_t row0, rows, qrows, hsplit;
    int32_t nh, ndense, dense0, c_exp;
    int32_t ds0, nds, pad[2];
};
static_assert(sizeof(RowTile) == 48, "RowTile layout");
// A dense diagonal block's part in a row tile: value (tile row r, column k)
// at dense[off + k * ld + r], x entries from xcol.
struct TileDense {
    int64_t off;
    int32_t ld, cols, xcol, pad;
};
static_assert(sizeof(TileDense) == 24, "TileDense layout");
// One warp's unit of row-side work: rows 16q .. 16q + 15 of a tile over the
// k-pairs kp = h, h + H, ... (nkps of them; B rows from slot0; digit groups
// from code_off; the tile's k axis has K slots), streamed in nsteps pipeline
// steps described by row_steps[step0 ..] (k-pairs | code bytes / 256 << 8 |
// the k-pairs' common info byte << 16 | 1 << 24 when the step is uniform: one
// info byte, every k-pair inside the k axis).
struct RowUnit {
    int32_t tile, q, h, H;
    int32_t nkps, K, slot0, nsteps;
    int64_t code_off, kp_off;
    int32_t step0, pad[3];
};
static_assert(sizeof(RowUnit) == 64, "RowUnit layout");

// A row-side B row slot: its component (-1: padding past the tile's k axis)
// and (split row + 1) << 8 | width (split row: the component's row in the
// partial sums of a split column task, as split_id * 33 + row; 0: unsplit).
struct SlotRec {
    int32_t comp, info;
};

// Bytes of one column-side shared-memory stage (code groups and x rows of
// the step's chunks); one row-side stage (code groups and B rows).  Two
// stages per warp, eight warps per CTA and two CTAs per SM: 6144-byte stages
// are the largest that fit (measured: larger stages cut the per-step costs;
// 7168-byte row stages gained nothing more).
constexpr int kColSlotBytes = 6144;
constexpr int kRowSlotBytes = 6144;
// Longest run of chunks one column unit walks.
constexpr int kMaxPartChunks = 16;
// Columns of a dense block in one column-side dense unit (one slice).
constexpr int kDenseCols = 16;
// Exponent offset of a row tile without nonzero components.
constexpr int32_t kNoExp = -4000;

// Digit planes of a width-w code, and whether its top plane is a nibble.
inline int code_planes(int w) { return (w + 7) / 8; }
inline bool top_is_nibble(int w) { return w - 8 * (code_planes(w) - 1) <= 4; }

// Byte offsets of each section inside the device arena.
struct Sections {
    size_t perm, iperm, lr, dd, comp_w, comp_s, tasks, task_rec, task_dest, qcodes, pcodes, dense, tiles, tdense, units,
        kp_info, slot_rec, row_steps, comp_sl, comp_sr;
    size_t total;
};

struct Layout {
    uint64_t order = 0;
    int32_t n_lr = 0, n_dense = 0, n_comp = 0, n_tiles = 0, n_chunks = 0;
    int32_t n_tasks = 0, n_split = 0, max_parts = 1;
    int32_t n_units = 0, n_slots = 0, n_tdense = 0, n_dest = 0, n_dslices = 0;
    std::vector<uint8_t> arena;  // host image of the device arena
    Sections sec{};
    double bound = 0;
    // traffic model (reference word counts) and stored sizes
    uint64_t code_bytes = 0, left_code_bytes = 0, right_code_bytes = 0, scale_bytes = 0,
             dense_bytes = 0, flops = 0;
    uint64_t stored_q_bytes = 0, stored_p_bytes = 0;
};

Layout build_layout(const HostMatrix& m);

// Words of the bit string of `rows` codes of width w.
inline uint64_t words_for_bits(uint64_t rows, int w) { return (rows * uint64_t(w) + 31) / 32; }

}  // namespace qhg
