// Resident layout of the multi-right-hand-side precision form (host side,
// CUDA-free, unit-testable on the CPU).
//
// The precision form applies the same quantized H-matrix to p right-hand
// sides at once on the 5th-generation tensor cores (tcgen05.mma, f16
// operands, FP32 accumulators in tensor memory):
//
//   column side  T = Q^T X per block column: M = 128 components of the blocks
//                that share a column range, K = 64 entries per chunk, N = 3p
//                (hi/mid/lo f16 limbs of every right-hand side);
//   row side     y = P U per 128-row tile: K = the components of every block
//                that meets the tile (64 per chunk), N = 3p limbs of U; the
//                dense diagonal blocks enter the same tile as f16 limb tiles
//                against the limbs of x.
//
// Codes are stored as base-256 digit planes of one byte per entry: a code c
// on P = ceil(w/8) planes has the unsigned lower digits (c >> 8m) & 255,
// m < P-1, and the signed top digit c >> 8(P-1) (two's complement byte).  The
// device turns plane m's digit d into an exact f16 d * 2^(8m + b) -- column
// side b = -24, row side b = -8(P-1) (top plane at 2^0), subnormal for the
// lowest plane of a 32-bit code -- so that all planes of a chunk accumulate
// into one FP32 sum equal to 2^b * sum_i c_i v_i up to FP32 rounding.  A chunk's codes all use the planes of its widest code
// (narrower codes sign-extended); components are sorted by width so chunks
// are nearly uniform.
#pragma once

#include <cstdint>
#include <vector>

#include "layout.hpp"

namespace qhg {

constexpr int kPfM = 128;        // MMA rows: components (column side) or matrix rows (row side)
constexpr int kPfK = 64;         // K entries of one chunk: one 128-byte row of f16 (one swizzle atom)
constexpr int kPfMaxRhs = 64;    // right-hand sides of one pass: N = 3p <= 192
constexpr int kPfPlaneBytes = kPfM * kPfK;  // one digit plane of a full chunk (8 KB)
constexpr int kPfTileBytes = kPfM * kPfK * 2;  // one f16 operand tile (16 KB, 128B-swizzled)

// A column-side work item: components [comp0, comp0 + count) (count <= 128,
// rows of the MMA tile) of blocks sharing one column range.  Its K axis is the
// clustered entries e_base + [0, 64 nkc) with e_base = col0 rounded down to a
// multiple of 8 (the x-limb tensor copies start on 16-byte boundaries);
// entries outside the range hold code 0.  Chunk kc, plane m: 128 rows x 64
// digit bytes at a_off + (kc * planes + m) * 8192 (row j = component j).
struct PfColItem {
    int64_t a_off;
    int32_t e_base, nkc, planes, count;
    int32_t comp0, pad;
};
static_assert(sizeof(PfColItem) == 32, "PfColItem layout");

// One component of a column item: s^P s^Q, and the row-side slots its u
// feeds (dests[dest0 .. dest0 + ndest)); a dest word is slot | (P - 1) << 28
// with P the digit planes of the row chunk holding the slot (the row side
// scales u by 256^(P-1) there, so that u' of every width shares one range).
struct PfComp {
    double scale;
    int32_t dest0, ndest;
};
static_assert(sizeof(PfComp) == 16, "PfComp layout");

// A row-side work item: K split `h` of the 128-row tile `tile` (clustered
// rows [row0, row0 + rows)), chunks [chunk0, chunk0 + nchunks); its FP64
// partial sums go to partial slot `part`.  Dense limb tiles of the tile are
// scaled by 2^-dense_exp.  u_beta: the item's own bound on its slots' u (as
// PfLayout::u_beta, over this item's slots only), so that the limbs of U'
// carry full precision whatever the other items' magnitudes.
struct PfRowItem {
    int32_t tile, row0, rows, part;
    int32_t chunk0, nchunks, dense_exp, u_beta;
};
static_assert(sizeof(PfRowItem) == 32, "PfRowItem layout");

// A row-side chunk.  kind 0 (low rank): slots [b, b + 64) of U (nvalid of them
// real; U of the others is read as 0) against `planes` digit planes of P at
// a_off, each of 64 digit bytes per stored row; half 0 stores all 128 tile
// rows, half 1 only rows 0..63, half 2 only rows 64..127 (the other rows are
// zero).  The chunk's plane m holds digits of weight 2^(8(m - P + 1)) (top plane
// 2^0): the codes times 2^(-8(P-1)), against u 256^(P-1) of its slots.
// kind 1 (dense): three pre-swizzled f16 limb tiles of a dense block
// part (3 x 16 KB at a_off) against the x limbs of clustered entries
// [b, b + 64) (b a multiple of 8).
struct PfRowChunk {
    int64_t a_off;
    int32_t b;
    uint8_t kind, planes, half, nvalid;
};
static_assert(sizeof(PfRowChunk) == 16, "PfRowChunk layout");

struct PfSections {
    size_t perm, col_items, comps, dests, row_items, chunks, col_sched, row_sched, qraw, praw, total;
};

struct PfLayout {
    uint64_t order = 0;
    int32_t n_col_items = 0, n_comp = 0, n_dests = 0, n_row_items = 0, n_chunks = 0, n_tiles = 0;
    int32_t n_parts = 0, n_slots = 0;
    int32_t grid = 0;  // persistent CTAs the schedules are built for
    // Layout-time bound on the row side's u operand: for every component j and
    // every destination chunk of P planes, |u_j| 256^(P-1) < 2^u_beta max|x|,
    // so the per-column scale of U' needs no pass over u.  The largest of the
    // row items' own bounds (PfRowItem::u_beta <= u_beta).
    int32_t u_beta = 0;
    double bound = 0;
    std::vector<uint8_t> arena;
    PfSections sec{};
    // per-tile partial slots: part p of tile t is partial index t_part0[t] + h
    std::vector<int32_t> tile_part0;
    // traffic model (packed reference bytes) and stored sizes
    uint64_t code_bytes = 0, scale_bytes = 0, dense_bytes = 0;
    uint64_t stored_q = 0, stored_p = 0, stored_dense = 0;
    uint64_t mma_col = 0, mma_row = 0;  // M x K elements streamed through the MMAs per pass
};

// Build the precision-form layout of a matrix; `grid` is the number of
// persistent CTAs whose static schedules are stored with it, and
// `row_items_per_cta` (default 3) how many row items (K splits of the 128-row
// tiles) each CTA gets on average -- the two schedule parameters the batching
// form's autotuner chooses.
PfLayout build_pf_layout(const HostMatrix& m, int grid, double row_items_per_cta = 0.0);

}  // namespace qhg
