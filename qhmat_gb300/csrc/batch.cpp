// Block-diagonal concatenation of independent matrices (the batching form).
//
// A batch of H-matrices A_1 .. A_M is applied as one block-diagonal matrix
// diag(A_1, .., A_M): its blocks are every matrix's blocks shifted to the
// matrix's offset, so one persistent launch of the column and row kernels
// walks the blocks of all of them (uneven sizes, ranks and widths), and each
// matrix's rows of y depend only on its own blocks and x.  Each matrix starts
// on a multiple of `align` rows, so that no 128-row tile and no column chunk
// spans two matrices.
#include "batch.hpp"

#include <stdexcept>

namespace qhg {

HostMatrix concat_block_diagonal(const std::vector<HostMatrix>& ms, uint64_t align, std::vector<uint64_t>& offsets) {
    if (ms.empty()) throw std::invalid_argument("empty batch");
    if (align == 0) align = 1;
    HostMatrix S;
    offsets.clear();
    uint64_t o = 0;
    for (const auto& m : ms) {
        offsets.push_back(o);
        o += (m.order + align - 1) / align * align;
    }
    S.order = o;
    S.permutation.resize(size_t(o));
    for (uint64_t r = 0; r < o; ++r) S.permutation[size_t(r)] = r;  // padding rows map to themselves
    for (size_t k = 0; k < ms.size(); ++k) {
        const HostMatrix& m = ms[k];
        const uint64_t off = offsets[k];
        for (uint64_t i = 0; i < m.order; ++i) S.permutation[size_t(off + i)] = off + m.permutation[size_t(i)];
        const uint64_t comp_base = S.width.size(), dense_base = S.dense.size();
        const uint64_t lw = S.left_words.size(), rw = S.right_words.size();
        for (const auto& b : m.blocks) {
            HostMatrix::Block c = b;
            c.row0 += off;
            c.row1 += off;
            c.col0 += off;
            c.col1 += off;
            c.comp0 += comp_base;
            c.dense_off += dense_base;
            S.blocks.push_back(c);
        }
        S.width.insert(S.width.end(), m.width.begin(), m.width.end());
        S.left_scale.insert(S.left_scale.end(), m.left_scale.begin(), m.left_scale.end());
        S.right_scale.insert(S.right_scale.end(), m.right_scale.begin(), m.right_scale.end());
        for (uint64_t v : m.left_off) S.left_off.push_back(v + lw);
        for (uint64_t v : m.right_off) S.right_off.push_back(v + rw);
        S.left_words.insert(S.left_words.end(), m.left_words.begin(), m.left_words.end());
        S.right_words.insert(S.right_words.end(), m.right_words.begin(), m.right_words.end());
        S.dense.insert(S.dense.end(), m.dense.begin(), m.dense.end());
    }
    return S;
}

}  // namespace qhg
