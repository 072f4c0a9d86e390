// QHMAT001 ingestion and construction of the resident device layout.
//
// The file format is the reference's (src/qhmat/io.cpp:139-163, little-endian,
// FNV-1a-64 trailer); the checks and their messages follow HMatrix::load
// (io.cpp:173-257) so that a caller switching from the reference sees the same
// errors.  The parser below is written from the format description, not from
// the reference's Reader class.
#include "layout.hpp"

#include "../../include/qhmat_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <utility>

namespace qhg {
namespace {

constexpr uint64_t kFnvOffset = kFnvOffsetBasis;
constexpr uint64_t kFnvPrime = kFnvPrimeValue;

// Cursor over the image.  `avail` counts bytes before the 8-byte trailer.
class Cursor {
public:
    Cursor(const uint8_t* p, size_t len) : p_(p), len_(len) {
        if (len < 24) throw runtime_error("truncated qhmat file");
        avail_ = len - 8;
    }
    uint64_t avail() const { return avail_ - pos_; }
    void need(uint64_t count, uint64_t width, const char* what = "truncated qhmat payload") const {
        if (width != 0 && count > avail() / width) throw runtime_error(what);
    }
    const uint8_t* take(uint64_t n) {
        if (n > avail()) throw runtime_error("truncated qhmat file");
        const uint8_t* q = p_ + pos_;
        pos_ += n;
        return q;
    }
    uint8_t u8() { return *take(1); }
    uint64_t u64() {
        const uint8_t* q = take(8);
        uint64_t v = 0;
        for (int i = 7; i >= 0; --i) v = (v << 8) | q[i];
        return v;
    }
    double f64() {
        uint64_t b = u64();
        double d;
        std::memcpy(&d, &b, 8);
        return d;
    }
    void u32s(uint32_t* out, uint64_t n) {
        const uint8_t* q = take(4 * n);
        for (uint64_t i = 0; i < n; ++i)
            out[i] = uint32_t(q[4 * i]) | uint32_t(q[4 * i + 1]) << 8 |
                     uint32_t(q[4 * i + 2]) << 16 | uint32_t(q[4 * i + 3]) << 24;
    }
    void f64s(double* out, uint64_t n) {
        for (uint64_t i = 0; i < n; ++i) out[i] = f64();
    }
    void finish() const {
        if (pos_ != avail_) throw runtime_error("trailing qhmat data");
        uint64_t h = kFnvOffset;
        for (size_t i = 0; i < avail_; ++i) h = (h ^ p_[i]) * kFnvPrime;
        uint64_t stored = 0;
        for (int i = 7; i >= 0; --i) stored = (stored << 8) | p_[avail_ + i];
        if (stored != h) throw runtime_error("qhmat checksum mismatch");
    }

private:
    const uint8_t* p_;
    size_t len_;
    uint64_t avail_ = 0, pos_ = 0;
};

uint64_t words_for(uint64_t rows, int bits) { return (rows * uint64_t(bits) + 31) / 32; }

void check_permutation(const std::vector<uint64_t>& perm) {
    std::vector<uint8_t> seen(perm.size(), 0);
    for (uint64_t v : perm) {
        if (v >= perm.size() || seen[v]) throw invalid_argument("permutation is not a bijection");
        seen[v] = 1;
    }
}

void check_rectangle(const HostMatrix::Block& b, uint64_t order) {
    if (!(b.row0 < b.row1 && b.row1 <= order && b.col0 < b.col1 && b.col1 <= order))
        throw invalid_argument("invalid block rectangle");
    const bool same = b.row0 == b.col0 && b.row1 == b.col1;
    const bool disjoint = b.row1 <= b.col0 || b.col1 <= b.row0;
    if (b.dense ? !same : !disjoint)
        throw invalid_argument(
            "only diagonal blocks may be dense; factorized blocks must be off-diagonal");
}

// HMatrix::finalize: the column intervals of the blocks covering each
// elementary row slab tile [0, order) exactly.
void check_cover(const HostMatrix& m) {
    if (m.blocks.empty()) throw invalid_argument("matrix has no blocks");
    std::vector<uint64_t> bounds{0, m.order};
    for (const auto& b : m.blocks) {
        bounds.push_back(b.row0);
        bounds.push_back(b.row1);
    }
    std::sort(bounds.begin(), bounds.end());
    bounds.erase(std::unique(bounds.begin(), bounds.end()), bounds.end());
    // Sweep: blocks sorted by row0; active set per slab.
    std::vector<uint32_t> by_row(m.blocks.size());
    std::iota(by_row.begin(), by_row.end(), 0u);
    std::sort(by_row.begin(), by_row.end(),
              [&](uint32_t a, uint32_t b) { return m.blocks[a].row0 < m.blocks[b].row0; });
    std::vector<uint32_t> active;
    size_t next = 0;
    std::vector<std::pair<uint64_t, uint64_t>> iv;
    for (size_t s = 0; s + 1 < bounds.size(); ++s) {
        const uint64_t r = bounds[s];
        while (next < by_row.size() && m.blocks[by_row[next]].row0 <= r) active.push_back(by_row[next++]);
        active.erase(std::remove_if(active.begin(), active.end(),
                                    [&](uint32_t b) { return m.blocks[b].row1 <= r; }),
                     active.end());
        iv.clear();
        for (uint32_t b : active) iv.emplace_back(m.blocks[b].col0, m.blocks[b].col1);
        std::sort(iv.begin(), iv.end());
        uint64_t end = 0;
        for (const auto& p : iv) {
            if (p.first != end) throw invalid_argument("block partition has a gap or overlap");
            end = p.second;
        }
        if (end != m.order) throw invalid_argument("block partition does not cover the matrix");
    }
}

}  // namespace

double HostMatrix::reconstruction_bound() const {
    double bound = 0.0;
    for (const auto& b : blocks) bound = std::max(bound, b.truncation_error + b.quantization_bound);
    return bound;
}

HostMatrix parse_qhmat(const uint8_t* bytes, size_t len) {
    Cursor c(bytes, len);
    HostMatrix m;
    const uint8_t* magic = c.take(8);
    if (std::memcmp(magic, "QHMAT001", 8) != 0) throw runtime_error("invalid qhmat file magic");
    if (c.u64() != 1) throw runtime_error("unsupported qhmat file version");
    const uint64_t order = c.u64(), count = c.u64();
    if (!order || !count || order > c.avail() / 8)
        throw runtime_error("invalid qhmat file dimensions");
    m.order = order;
    m.permutation.resize(order);
    for (auto& v : m.permutation) v = c.u64();
    check_permutation(m.permutation);
    if (count > c.avail() / 34) throw runtime_error("invalid qhmat block count");
    m.blocks.reserve(count);
    for (uint64_t k = 0; k < count; ++k) {
        HostMatrix::Block b;
        b.row0 = c.u64();
        b.row1 = c.u64();
        b.col0 = c.u64();
        b.col1 = c.u64();
        const uint8_t adm = c.u8(), dense = c.u8();
        if (adm > 1 || dense > 1) throw runtime_error("invalid qhmat block flag");
        b.admissible = adm == 1;
        b.dense = dense == 1;
        check_rectangle(b, order);
        const uint64_t rows = b.row1 - b.row0, cols = b.col1 - b.col0;
        if (b.dense) {
            if (cols > std::numeric_limits<uint64_t>::max() / rows)
                throw runtime_error("dense block size overflow");
            const uint64_t total = rows * cols;
            c.need(total, 8);
            b.dense_off = m.dense.size();
            m.dense.resize(m.dense.size() + total);
            c.f64s(m.dense.data() + b.dense_off, total);
            for (uint64_t i = 0; i < total; ++i)
                if (!std::isfinite(m.dense[b.dense_off + i]))
                    throw runtime_error("nonfinite dense value");
        } else {
            const uint64_t rank = c.u64(), menu = c.u64();
            if (rank > std::min(rows, cols) || menu == 0 || menu > 31)
                throw runtime_error("invalid qhmat rank or precision menu");
            b.truncation_error = c.f64();
            b.quantization_bound = c.f64();
            if (!std::isfinite(b.truncation_error) || b.truncation_error < 0 ||
                !std::isfinite(b.quantization_bound) || b.quantization_bound < 0)
                throw runtime_error("invalid qhmat error bound");
            c.need(rank, 17);
            b.rank = rank;
            b.comp0 = m.width.size();
            for (uint64_t j = 0; j < rank; ++j) {
                const uint8_t w = c.u8();
                if (w < 2 || w > 32) throw runtime_error("invalid qhmat bit width");
                m.width.push_back(w);
            }
            const size_t s0 = m.left_scale.size();
            m.left_scale.resize(s0 + rank);
            m.right_scale.resize(s0 + rank);
            c.f64s(m.left_scale.data() + s0, rank);
            c.f64s(m.right_scale.data() + s0, rank);
            for (uint64_t j = 0; j < rank; ++j) {
                const double l = m.left_scale[s0 + j], r = m.right_scale[s0 + j];
                if (!std::isfinite(l) || l < 0 || !std::isfinite(r) || r < 0)
                    throw runtime_error("invalid qhmat scale");
            }
            uint64_t lw = 0, rw = 0;
            for (uint64_t j = 0; j < rank; ++j) {
                m.left_off.push_back(m.left_words.size() + lw);
                m.right_off.push_back(m.right_words.size() + rw);
                lw += words_for(rows, m.width[b.comp0 + j]);
                rw += words_for(cols, m.width[b.comp0 + j]);
            }
            c.need(lw + rw, 4);
            const size_t l0 = m.left_words.size(), r0 = m.right_words.size();
            m.left_words.resize(l0 + lw);
            m.right_words.resize(r0 + rw);
            c.u32s(m.left_words.data() + l0, lw);
            c.u32s(m.right_words.data() + r0, rw);
        }
        m.blocks.push_back(b);
    }
    c.finish();
    check_cover(m);
    return m;
}

void validate(const HostMatrix& m) {
    if (m.order == 0 || m.permutation.size() != m.order)
        throw invalid_argument("invalid matrix order/permutation");
    check_permutation(m.permutation);
    for (const auto& b : m.blocks) {
        check_rectangle(b, m.order);
        const uint64_t rows = b.row1 - b.row0, cols = b.col1 - b.col0;
        if (b.dense) {
            if (b.dense_off + rows * cols > m.dense.size())
                throw invalid_argument("dense block shape mismatch");
            for (uint64_t i = 0; i < rows * cols; ++i)
                if (!std::isfinite(m.dense[b.dense_off + i]))
                    throw invalid_argument("nonfinite dense block");
        } else {
            if (b.rank > std::min(rows, cols) || b.comp0 + b.rank > m.width.size())
                throw invalid_argument("factor dimensions do not match block rank");
            for (uint64_t j = 0; j < b.rank; ++j) {
                const uint64_t c = b.comp0 + j;
                const int w = m.width[c];
                if (w < 2 || w > 32) throw invalid_argument("bit width must be in [2, 32]");
                if (!std::isfinite(m.left_scale[c]) || m.left_scale[c] < 0 ||
                    !std::isfinite(m.right_scale[c]) || m.right_scale[c] < 0)
                    throw invalid_argument("invalid scale");
                if (m.left_off[c] + words_for(rows, w) > m.left_words.size() ||
                    m.right_off[c] + words_for(cols, w) > m.right_words.size())
                    throw invalid_argument("packed factor offsets out of range");
            }
        }
    }
    check_cover(m);
}

namespace {

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

template <class T>
T* at(std::vector<uint8_t>& arena, size_t off) {
    return reinterpret_cast<T*>(arena.data() + off);
}

}  // namespace

Layout build_layout(const HostMatrix& m) {
    Layout L;
    L.order = m.order;
    L.bound = m.reconstruction_bound();
    if (m.order >= (1ull << 31)) throw overflow_error("matrix order too large for the device layout");
    if (m.width.size() >= (1ull << 31)) throw overflow_error("too many components for the device layout");
    if (m.left_words.size() >= (1ull << 32) || m.right_words.size() >= (1ull << 32))
        throw overflow_error("packed factors too large for the device layout");

    std::vector<LowRankDesc> lr;
    std::vector<DenseDesc> dd;
    std::vector<int32_t> block_item(m.blocks.size());  // item code per block
    for (size_t k = 0; k < m.blocks.size(); ++k) {
        const auto& b = m.blocks[k];
        const int32_t r0 = int32_t(b.row0), mm = int32_t(b.row1 - b.row0);
        const int32_t c0 = int32_t(b.col0), nn = int32_t(b.col1 - b.col0);
        if (b.dense) {
            block_item[k] = -1 - int32_t(dd.size());
            dd.push_back({r0, mm, c0, nn, int64_t(b.dense_off)});
            L.dense_bytes += 8ull * uint64_t(mm) * uint64_t(nn);
            L.flops += 2ull * uint64_t(mm) * uint64_t(nn);
        } else {
            block_item[k] = int32_t(lr.size());
            lr.push_back({r0, mm, c0, nn, int32_t(b.rank), int32_t(b.comp0)});
            L.scale_bytes += 16ull * b.rank;
            L.flops += 2ull * b.rank * uint64_t(mm + nn);
            for (uint64_t j = 0; j < b.rank; ++j) {
                const int w = m.width[b.comp0 + j];
                L.code_bytes += 4ull * (words_for(uint64_t(mm), w) + words_for(uint64_t(nn), w));
            }
        }
    }
    L.n_lr = int32_t(lr.size());
    L.n_dense = int32_t(dd.size());
    L.n_comp = int32_t(m.width.size());
    L.n_chunks = int32_t((m.order + kChunk - 1) / kChunk);

    // Column side: low-rank blocks with rank > 0, heaviest first.
    std::vector<int32_t> a_order;
    for (int32_t i = 0; i < L.n_lr; ++i)
        if (lr[i].rank > 0) a_order.push_back(i);
    std::stable_sort(a_order.begin(), a_order.end(), [&](int32_t a, int32_t b) {
        return int64_t(lr[a].rank) * lr[a].n > int64_t(lr[b].rank) * lr[b].n;
    });
    L.n_a = int32_t(a_order.size());

    // Row side: elementary slabs (finalize's row boundaries), each cut into
    // tiles of at most kTileRows rows.  A slab's items are the blocks covering
    // it, in insertion order.
    std::vector<uint64_t> bounds{0, m.order};
    for (const auto& b : m.blocks) {
        bounds.push_back(b.row0);
        bounds.push_back(b.row1);
    }
    std::sort(bounds.begin(), bounds.end());
    bounds.erase(std::unique(bounds.begin(), bounds.end()), bounds.end());
    const size_t n_slabs = bounds.size() - 1;
    std::vector<std::vector<int32_t>> slab_items(n_slabs);
    for (size_t k = 0; k < m.blocks.size(); ++k) {
        const auto& b = m.blocks[k];
        size_t s = size_t(std::lower_bound(bounds.begin(), bounds.end(), b.row0) - bounds.begin());
        for (; s < n_slabs && bounds[s] < b.row1; ++s) slab_items[s].push_back(block_item[k]);
    }
    std::vector<int32_t> items;
    std::vector<RowTile> tiles;
    std::vector<int64_t> tile_work;
    for (size_t s = 0; s < n_slabs; ++s) {
        const int32_t i0 = int32_t(items.size());
        int64_t comp_sum = 0, work_per_row = 0;
        for (int32_t it : slab_items[s]) {
            items.push_back(it);
            if (it >= 0) {
                comp_sum += lr[it].rank;
                work_per_row += lr[it].rank;
            } else {
                work_per_row += dd[-1 - it].n;
            }
        }
        const int32_t i1 = int32_t(items.size());
        L.max_tile_items_comp = std::max<int32_t>(L.max_tile_items_comp, int32_t(comp_sum));
        for (uint64_t r = bounds[s]; r < bounds[s + 1]; r += kTileRows) {
            const int32_t rows = int32_t(std::min<uint64_t>(kTileRows, bounds[s + 1] - r));
            tiles.push_back({int32_t(r), rows, i0, i1});
            tile_work.push_back(work_per_row * rows);
        }
    }
    std::vector<int32_t> torder(tiles.size());
    std::iota(torder.begin(), torder.end(), 0);
    std::stable_sort(torder.begin(), torder.end(),
                     [&](int32_t a, int32_t b) { return tile_work[a] > tile_work[b]; });
    std::vector<RowTile> tiles_sorted(tiles.size());
    for (size_t i = 0; i < tiles.size(); ++i) tiles_sorted[i] = tiles[torder[i]];
    L.n_tiles = int32_t(tiles.size());
    L.n_items = int32_t(items.size());

    // Arena sections, each 256-byte aligned.
    Sections& S = L.sec;
    size_t off = 0;
    auto place = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + std::max<size_t>(bytes, 1), 256);
        return o;
    };
    const size_t C = m.width.size();
    S.perm = place(4 * m.order);
    S.lr = place(sizeof(LowRankDesc) * lr.size());
    S.dd = place(sizeof(DenseDesc) * dd.size());
    S.comp_w = place(C);
    S.comp_s = place(8 * C);
    S.comp_qoff = place(4 * C);
    S.comp_poff = place(4 * C);
    S.qwords = place(4 * m.right_words.size() + 16);
    S.pwords = place(4 * m.left_words.size() + 16);
    S.dense = place(8 * m.dense.size());
    S.a_order = place(4 * a_order.size());
    S.tiles = place(sizeof(RowTile) * tiles.size());
    S.items = place(4 * items.size());
    S.total = off;

    L.arena.assign(S.total, 0);
    auto& A = L.arena;
    for (uint64_t i = 0; i < m.order; ++i) at<int32_t>(A, S.perm)[i] = int32_t(m.permutation[i]);
    if (!lr.empty()) std::memcpy(at<LowRankDesc>(A, S.lr), lr.data(), sizeof(LowRankDesc) * lr.size());
    if (!dd.empty()) std::memcpy(at<DenseDesc>(A, S.dd), dd.data(), sizeof(DenseDesc) * dd.size());
    for (size_t c = 0; c < C; ++c) {
        at<uint8_t>(A, S.comp_w)[c] = m.width[c];
        // One rounding: s_P * s_Q.  In exact arithmetic the block contribution
        // sum_j (s_P c_P)(sum_k s_Q c_Q x) equals sum_j c_P (s_P s_Q) sum_k c_Q x.
        at<double>(A, S.comp_s)[c] = m.left_scale[c] * m.right_scale[c];
        at<uint32_t>(A, S.comp_qoff)[c] = uint32_t(m.right_off[c]);
        at<uint32_t>(A, S.comp_poff)[c] = uint32_t(m.left_off[c]);
    }
    if (!m.right_words.empty())
        std::memcpy(A.data() + S.qwords, m.right_words.data(), 4 * m.right_words.size());
    if (!m.left_words.empty())
        std::memcpy(A.data() + S.pwords, m.left_words.data(), 4 * m.left_words.size());
    if (!m.dense.empty()) std::memcpy(A.data() + S.dense, m.dense.data(), 8 * m.dense.size());
    if (!a_order.empty()) std::memcpy(A.data() + S.a_order, a_order.data(), 4 * a_order.size());
    if (!tiles_sorted.empty())
        std::memcpy(A.data() + S.tiles, tiles_sorted.data(), sizeof(RowTile) * tiles_sorted.size());
    if (!items.empty()) std::memcpy(A.data() + S.items, items.data(), 4 * items.size());
    return L;
}

}  // namespace qhg

extern "C" uint64_t qh_fnv1a64(const void* bytes, size_t len) {
    const auto* p = static_cast<const uint8_t*>(bytes);
    uint64_t h = qhg::kFnvOffsetBasis;
    for (size_t i = 0; i < len; ++i) h = (h ^ p[i]) * qhg::kFnvPrimeValue;
    return h;
}
