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
#include <cstdlib>
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

// Copy the bit string [bit0, bit0 + nbits) of a run of `run_words` words to
// out[0 .. ceil(nbits/32)), starting at a fresh word; bits past the string
// (or past the run) are zero.
// Code i of a component's run: bits [i*w, i*w + w), LSB-first, sign-extended
// -- the field HMatrix::decode reads (src/qhmat/core.cpp:269-282).
int32_t code_of(const uint32_t* run, uint64_t i, int w) {
    const uint64_t pos = i * uint64_t(w), wi = pos >> 5, off = pos & 31;
    uint64_t v = run[wi];
    if (off + uint64_t(w) > 32) v |= uint64_t(run[wi + 1]) << 32;
    const uint64_t f = (v >> off) & ((uint64_t(1) << w) - 1);
    return int32_t(int64_t(f << (64 - w)) >> (64 - w));
}

// Offset code u = c + 2^(w-1) in [0, 2^w).
inline uint32_t offset_code(int32_t c, int w) { return uint32_t(int64_t(c) + (int64_t(1) << (w - 1))); }

// Position of k-block kb entry e (0..15) inside a fragment row: thread t and
// slot s (0..3: entries 2t, 2t+1, 2t+8, 2t+9).
inline void frag_pos(int e, int& t, int& slot) {
    t = (e & 7) >> 1;
    slot = (e & 1) | ((e >> 3) << 1);
}

// Store digit d of (k-block kb, entry e) into a group row at `row` (32 bytes
// for a byte group, 16 for a nibble group).
inline void put_digit(uint8_t* row, bool nib, int kb, int e, uint32_t d) {
    int t, slot;
    frag_pos(e, t, slot);
    if (!nib) {
        row[8 * t + 4 * kb + slot] = uint8_t(d);
    } else {
        // register k = 2kb + (slot >> 1) of the pair: low half nibble k, high
        // half nibble k + 4
        const int nibble = 2 * kb + (slot >> 1) + 4 * (slot & 1);
        uint32_t w;
        std::memcpy(&w, row + 4 * t, 4);
        w |= (d & 15u) << (4 * nibble);
        std::memcpy(row + 4 * t, &w, 4);
    }
}

// Longest run of chunks one column unit walks: kMaxPartChunks, or fewer when
// the environment variable QHMAT_GB300_PART_CHUNKS (1 .. kMaxPartChunks) asks
// for it -- a test knob that sends short tasks through the split-task path
// (partial sums combined by the last part); results are bitwise the same.
int32_t part_chunks_setting() {
    const char* v = std::getenv("QHMAT_GB300_PART_CHUNKS");
    if (!v || !*v) return kMaxPartChunks;
    const long k = std::strtol(v, nullptr, 10);
    return int32_t(std::min<long>(kMaxPartChunks, std::max<long>(1, k)));
}

}  // namespace

Layout build_layout(const HostMatrix& m) {
    Layout L;
    const int32_t part_chunks = part_chunks_setting();
    L.order = m.order;
    L.bound = m.reconstruction_bound();
    if (m.order >= (1ull << 31)) throw overflow_error("matrix order too large for the device layout");
    if (m.width.size() >= (1ull << 31)) throw overflow_error("too many components for the device layout");

    std::vector<LowRankDesc> lr;
    std::vector<DenseDesc> dd;
    std::vector<int32_t> block_item(m.blocks.size());
    std::vector<size_t> block_of_lr;
    std::vector<double> dense_cm;  // column-major copies
    for (size_t k = 0; k < m.blocks.size(); ++k) {
        const auto& b = m.blocks[k];
        const int32_t r0 = int32_t(b.row0), mm = int32_t(b.row1 - b.row0);
        const int32_t c0 = int32_t(b.col0), nn = int32_t(b.col1 - b.col0);
        if (b.dense) {
            block_item[k] = -1 - int32_t(dd.size());
            dd.push_back({r0, mm, c0, nn, int64_t(dense_cm.size())});
            const double* src = m.dense.data() + b.dense_off;
            const size_t base = dense_cm.size();
            dense_cm.resize(base + size_t(mm) * size_t(nn));
            for (int32_t i = 0; i < mm; ++i)
                for (int32_t c = 0; c < nn; ++c) dense_cm[base + size_t(c) * mm + i] = src[size_t(i) * nn + c];
            L.dense_bytes += 8ull * uint64_t(mm) * uint64_t(nn);
            L.flops += 2ull * uint64_t(mm) * uint64_t(nn);
        } else {
            block_item[k] = int32_t(lr.size());
            lr.push_back({r0, mm, c0, nn, int32_t(b.rank), int32_t(b.comp0)});
            block_of_lr.push_back(k);
            L.scale_bytes += 16ull * b.rank;
            L.flops += 2ull * b.rank * uint64_t(mm + nn);
            for (uint64_t j = 0; j < b.rank; ++j) {
                const int w = m.width[b.comp0 + j];
                L.left_code_bytes += 4ull * words_for_bits(uint64_t(mm), w);
                L.right_code_bytes += 4ull * words_for_bits(uint64_t(nn), w);
            }
        }
    }
    L.code_bytes = L.left_code_bytes + L.right_code_bytes;
    L.n_lr = int32_t(lr.size());
    L.n_dense = int32_t(dd.size());
    L.n_comp = int32_t(m.width.size());
    L.n_chunks = int32_t((m.order + kChunk - 1) / kChunk);

    // ---- column side: tasks of <= 32 components sharing (col0, n, width).
    // beta[c]: |u_c| < 2^(xe - 1022 + beta[c]) for x whose exponent fields are
    // <= xe (|u| <= |s^P s^Q| * ||c^Q||_1 * max|x|, one binade of slack for
    // rounding); kNoExp when u is identically zero.
    std::vector<int32_t> beta(m.width.size(), kNoExp);
    struct Key {
        int32_t col0, n, w;
        bool operator<(const Key& o) const {
            if (col0 != o.col0) return col0 < o.col0;
            if (n != o.n) return n < o.n;
            return w < o.w;
        }
    };
    std::vector<std::pair<Key, int32_t>> comps;  // (key, component id), in block order
    for (const auto& d : lr)
        for (int32_t j = 0; j < d.rank; ++j)
            comps.push_back({{d.col0, d.n, int32_t(m.width[d.comp0 + j])}, d.comp0 + j});
    std::stable_sort(comps.begin(), comps.end(),
                     [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<ColTask> tasks;
    std::vector<TaskRec> task_rec;
    std::vector<int32_t> comp_part(m.width.size(), -1);  // row of a split task's partial sums, or -1
    std::vector<uint8_t> qcodes;
    int32_t n_split = 0;
    for (size_t i = 0; i < comps.size();) {
        size_t j = i;
        while (j < comps.size() && !(comps[i].first < comps[j].first) && !(comps[j].first < comps[i].first)) ++j;
        for (size_t t0 = i; t0 < j; t0 += 32) {
            const int32_t count = int32_t(std::min<size_t>(32, j - t0));
            const Key key = comps[t0].first;
            const int P = code_planes(key.w);
            const bool nibtop = top_is_nibble(key.w);
            const int32_t row_bytes = (P - 1) * 32 + (nibtop ? 16 : 32);  // one row, all planes
            const int32_t stride = count * row_bytes;
            const int32_t nchunks = (key.n + kColChunk - 1) / kColChunk;
            const int32_t comp_idx = int32_t(task_rec.size());
            for (int32_t l = 0; l < count; ++l) {
                const int32_t c = comps[t0 + l].second;
                // One rounding: s_P * s_Q.  In exact arithmetic the block contribution
                // sum_j (s_P c_P)(sum_k s_Q c_Q x) equals sum_j c_P (s_P s_Q) sum_k c_Q x.
                task_rec.push_back({c, key.w, m.left_scale[size_t(c)] * m.right_scale[size_t(c)]});
            }
            const size_t base = qcodes.size();  // multiple of 16 bytes
            qcodes.resize(base + size_t(nchunks) * size_t(stride), 0);
            for (int32_t l = 0; l < count; ++l) {
                const int32_t c = comps[t0 + l].second;
                const uint32_t* run = m.right_words.data() + m.right_off[size_t(c)];
                const int q = l / 16, r = l % 16;
                const int rows_q = std::min<int32_t>(16, count - 16 * q);
                double l1 = 0.0;
                for (int32_t ch = 0; ch < nchunks; ++ch) {
                    // group (q, mm) of chunk ch starts after the earlier M-tile's groups
                    size_t goff = base + size_t(ch) * size_t(stride) + size_t(q) * 16 * size_t(row_bytes);
                    for (int mm = 0; mm < P; ++mm) {
                        const bool nb = nibtop && mm == P - 1;
                        const size_t rb = nb ? 16 : 32;
                        uint8_t* row = qcodes.data() + goff + size_t(r) * rb;
                        for (int e = 0; e < kColChunk; ++e) {
                            // entries past the range hold code 0 (every digit
                            // of it reads as zero on the device)
                            const int64_t idx = int64_t(ch) * kColChunk + e;
                            const int32_t code = idx < key.n ? code_of(run, uint64_t(idx), key.w) : 0;
                            if (mm == 0) l1 += std::fabs(double(code));
                            const uint32_t u = offset_code(code, key.w);
                            put_digit(row, nb, e >> 4, e & 15, (u >> (8 * mm)) & (nb ? 15u : 255u));
                        }
                        goff += size_t(rows_q) * rb;
                    }
                }
                const double bound = l1 * std::fabs(m.left_scale[size_t(c)] * m.right_scale[size_t(c)]);
                if (bound > 0.0 && std::isfinite(bound)) beta[size_t(c)] = int32_t(std::ilogb(bound)) + 2;
            }
            const int32_t nparts = (nchunks + part_chunks - 1) / part_chunks;
            const int32_t split_id = nparts > 1 ? n_split++ : -1;
            if (split_id >= 0)
                for (int32_t l = 0; l < count; ++l) comp_part[size_t(comps[t0 + l].second)] = split_id * 33 + l;
            L.max_parts = std::max(L.max_parts, nparts);
            const int32_t cps = std::max<int32_t>(1, kColSlotBytes / (stride + kColChunk * 16));
            for (int32_t pt = 0; pt < nparts; ++pt) {
                ColTask T{};
                T.col0 = key.col0;
                T.n = key.n;
                T.count = count;
                T.width = key.w;
                T.off = int64_t(base);
                T.stride = stride;
                T.comp_idx = comp_idx;
                T.chunk0 = pt * part_chunks;
                T.nchunks = std::min(part_chunks, nchunks - T.chunk0);
                T.part = pt;
                T.nparts = nparts;
                T.split_id = split_id;
                T.cps = cps;
                tasks.push_back(T);
            }
        }
        i = j;
    }
    // heaviest units first
    std::stable_sort(tasks.begin(), tasks.end(), [](const ColTask& a, const ColTask& b) {
        return int64_t(a.nchunks) * (a.stride + 512) > int64_t(b.nchunks) * (b.stride + 512);
    });
    L.n_tasks = int32_t(tasks.size());
    L.n_split = n_split;
    L.stored_q_bytes = qcodes.size();

    // ---- row side: elementary slabs (finalize's row boundaries) cut into tiles.
    std::vector<uint64_t> bounds{0, m.order};
    for (const auto& b : m.blocks) {
        bounds.push_back(b.row0);
        bounds.push_back(b.row1);
    }
    std::sort(bounds.begin(), bounds.end());
    bounds.erase(std::unique(bounds.begin(), bounds.end()), bounds.end());
    const size_t n_slabs = bounds.size() - 1;
    std::vector<std::vector<int32_t>> slab_blocks(n_slabs);
    for (size_t k = 0; k < m.blocks.size(); ++k) {
        const auto& b = m.blocks[k];
        size_t s = size_t(std::lower_bound(bounds.begin(), bounds.end(), b.row0) - bounds.begin());
        for (; s < n_slabs && bounds[s] < b.row1; ++s) slab_blocks[s].push_back(int32_t(k));
    }
    std::vector<RowTile> tiles;
    std::vector<std::pair<int64_t, RowUnit>> units;  // (cost, unit)
    std::vector<uint8_t> pcodes;
    std::vector<uint8_t> kp_info;
    int64_t n_slots = 0;
    std::vector<TileDense> tdense;
    std::vector<SlotRec> slot_rec;   // each B row slot's component, split row and width
    std::vector<std::vector<std::pair<int32_t, int32_t>>> comp_dest(m.width.size());  // per component: (slot, tile)
    std::vector<uint32_t> row_steps; // pipeline steps of the row units
    struct RowComp {
        int w;
        int32_t comp;
        int32_t block;  // index into m.blocks
    };
    for (size_t s = 0; s < n_slabs; ++s) {
        for (uint64_t r = bounds[s]; r < bounds[s + 1]; r += kTileRows) {
            const int32_t rows = int32_t(std::min<uint64_t>(kTileRows, bounds[s + 1] - r));
            const int32_t ti = int32_t(tiles.size());
            RowTile T{};
            T.row0 = int32_t(r);
            T.rows = rows;
            T.dense0 = int32_t(tdense.size());
            std::vector<RowComp> kc;
            for (int32_t k : slab_blocks[s]) {
                const auto& b = m.blocks[size_t(k)];
                const int32_t rloc0 = int32_t(r - b.row0);
                if (b.dense) {
                    const DenseDesc& d = dd[size_t(-1 - block_item[size_t(k)])];
                    tdense.push_back({d.off + rloc0, d.m, d.n, d.col0, 0});
                    ++T.ndense;
                    continue;
                }
                for (uint64_t j = 0; j < b.rank; ++j)
                    kc.push_back({int(m.width[b.comp0 + j]), int32_t(b.comp0 + j), k});
            }
            std::stable_sort(kc.begin(), kc.end(), [](const RowComp& a, const RowComp& b) { return a.w > b.w; });
            const int32_t K = int32_t(kc.size());
            const int32_t Kp = (K + 31) / 32;
            T.qrows = (rows + 15) / 16;
            T.hsplit = kTileUnits / T.qrows;
            T.nh = std::min(T.hsplit, Kp);
            T.c_exp = kNoExp;
            for (const auto& c : kc) T.c_exp = std::max(T.c_exp, beta[size_t(c.comp)]);
            const int64_t kp_off = int64_t(kp_info.size());
            // per k-pair (widths non-increasing along k): the planes and top
            // digit bits of its widest code; narrower codes are written on
            // the same planes (sign-extended)
            std::vector<int> kplanes(static_cast<size_t>(Kp), 0), knib(static_cast<size_t>(Kp), 0),
                ktop(static_cast<size_t>(Kp), 0);
            for (int32_t kp = 0; kp < Kp; ++kp) {
                const int w = kc[size_t(32 * kp)].w;
                const int planes = code_planes(w), tb = w - 8 * (planes - 1);
                kplanes[size_t(kp)] = planes;
                knib[size_t(kp)] = top_is_nibble(w) ? 1 << (planes - 1) : 0;
                ktop[size_t(kp)] = tb;
                kp_info.push_back(uint8_t(planes | (top_is_nibble(w) ? 8 : 0) | ((tb - 1) << 4)));
            }
            // B row slots: k split h's k-pairs contiguously
            std::vector<int64_t> hslot(size_t(T.hsplit), 0);
            for (int32_t h = 0; h < T.nh; ++h) {
                hslot[size_t(h)] = n_slots;
                for (int32_t kp = h; kp < Kp; kp += T.hsplit) {
                    for (int e = 0; e < 32; ++e) {
                        const int32_t k = 32 * kp + e;
                        if (k < K) {
                            const int32_t c = kc[size_t(k)].comp;
                            slot_rec.push_back({c, ((comp_part[size_t(c)] + 1) << 8) | int32_t(m.width[size_t(c)])});
                            comp_dest[size_t(c)].push_back({int32_t(slot_rec.size() - 1), ti});
                        } else {
                            slot_rec.push_back({-1, 1});
                        }
                    }
                }
                n_slots += 32 * int64_t((Kp - h + T.hsplit - 1) / T.hsplit);
            }
            // streams (q, h): groups of 16 rows
            for (int32_t q = 0; q < T.qrows; ++q)
                for (int32_t h = 0; h < T.nh; ++h) {
                    RowUnit U{};
                    U.tile = ti;
                    U.q = q;
                    U.h = h;
                    U.H = T.hsplit;
                    U.nkps = (Kp - h + T.hsplit - 1) / T.hsplit;
                    U.K = K;
                    U.slot0 = int32_t(hslot[size_t(h)]);
                    U.code_off = int64_t(pcodes.size());
                    U.kp_off = kp_off;
                    int64_t bytes = 0;
                    // pipeline steps: consecutive k-pairs (digit groups and
                    // 512 bytes of B rows each) filling a row-side stage
                    U.step0 = int32_t(row_steps.size());
                    {
                        // a step whose k-pairs share one info byte and lie
                        // wholly inside the k axis is marked uniform (the
                        // kernel then dispatches once per step)
                        int sc = 0, sb = 0;
                        bool uni = true;
                        uint32_t uinfo = 0;
                        auto flush = [&]() {
                            row_steps.push_back(uint32_t(sc) | uint32_t(sb / 256) << 8 |
                                                (uni ? (uinfo << 16) | (1u << 24) : 0u));
                            sc = 0;
                            sb = 0;
                            uni = true;
                        };
                        for (int32_t kp = h; kp < Kp; kp += T.hsplit) {
                            int cb = 0;
                            for (int mm = 0; mm < kplanes[size_t(kp)]; ++mm) cb += ((knib[size_t(kp)] >> mm) & 1) ? 256 : 512;
                            if (sc && sb + cb + 512 * (sc + 1) > kRowSlotBytes) flush();
                            const uint32_t info = kp_info[size_t(kp_off + kp)];
                            if (sc == 0) uinfo = info;
                            if (info != uinfo || 32 * (kp + 1) > K) uni = false;
                            ++sc;
                            sb += cb;
                        }
                        if (sc) flush();
                    }
                    U.nsteps = int32_t(row_steps.size()) - U.step0;
                    for (int32_t kp = h; kp < Kp; kp += T.hsplit)
                        for (int mm = 0; mm < kplanes[size_t(kp)]; ++mm) {
                            const bool nb = (knib[size_t(kp)] >> mm) & 1;
                            const bool top = mm == kplanes[size_t(kp)] - 1;
                            const int64_t half = int64_t(1) << (ktop[size_t(kp)] - 1);
                            const size_t rb = nb ? 16 : 32;
                            const size_t g0 = pcodes.size();
                            pcodes.resize(g0 + 16 * rb, 0);
                            for (int rr = 0; rr < 16; ++rr) {
                                const int32_t tr = 16 * q + rr;  // tile row
                                if (tr >= rows) break;
                                uint8_t* row = pcodes.data() + g0 + size_t(rr) * rb;
                                for (int e = 0; e < 32; ++e) {
                                    const int32_t k = 32 * kp + e;
                                    if (k >= K) break;
                                    const RowComp& c = kc[size_t(k)];
                                    const auto& b = m.blocks[size_t(c.block)];
                                    const uint32_t* run = m.left_words.data() + m.left_off[size_t(c.comp)];
                                    const uint64_t br = r + uint64_t(tr) - b.row0;
                                    const int64_t code = code_of(run, br, c.w);
                                    const int64_t d = top ? (code >> (8 * mm)) + half : (code >> (8 * mm)) & 255;
                                    put_digit(row, nb, e >> 4, e & 15, uint32_t(d) & (nb ? 15u : 255u));
                                }
                            }
                            bytes += int64_t(16 * rb);
                        }
                    units.push_back({bytes + int64_t(U.nkps) * 512, U});
                }
            if (T.qrows * T.nh + T.ndense == 0) throw runtime_error("row tile without blocks");
            tiles.push_back(T);
        }
    }
    if (n_slots >= (int64_t(1) << 31)) throw overflow_error("too many row-side slots for the device layout");
    // heaviest units first: the warps take them round-robin
    std::stable_sort(units.begin(), units.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    std::vector<RowUnit> unit_list;
    for (const auto& u : units) unit_list.push_back(u.second);
    L.n_tiles = int32_t(tiles.size());
    for (const auto& R : tiles)
        if (R.c_exp < -32768 || R.c_exp > 32767) throw overflow_error("row tile exponent out of range");
    // per column task: the B rows its components feed (component row << 24)
    std::vector<TaskDest> task_dest;
    for (auto& T : tasks) {
        if (T.part == 0 || T.nparts == 1) {
            T.dest0 = int32_t(task_dest.size());
            std::vector<std::pair<int32_t, TaskDest>> lst;  // (tile, record)
            for (int32_t r = 0; r < T.count; ++r)
                for (const auto& [slot, ti] : comp_dest[size_t(task_rec[size_t(T.comp_idx + r)].comp)]) {
                    const int32_t ce = tiles[size_t(ti)].c_exp;
                    lst.push_back({ti, {slot, (r << 16) | int32_t(uint16_t(int16_t(ce)))}});
                }
            std::stable_sort(lst.begin(), lst.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            for (const auto& e : lst) task_dest.push_back(e.second);
            T.ndest = int32_t(task_dest.size()) - T.dest0;
        }
    }
    // parts of a split task share its list
    {
        std::vector<std::pair<int32_t, int32_t>> by_split(size_t(n_split), {0, 0});
        for (const auto& T : tasks)
            if (T.nparts > 1 && T.part == 0) by_split[size_t(T.split_id)] = {T.dest0, T.ndest};
        for (auto& T : tasks)
            if (T.nparts > 1) {
                T.dest0 = by_split[size_t(T.split_id)].first;
                T.ndest = by_split[size_t(T.split_id)].second;
            }
    }
    {
        size_t fed = 0;
        for (const auto& v : comp_dest) fed += v.size();
        if (fed != task_dest.size()) throw runtime_error("internal: a row-side B row has no column task");
    }
    L.n_dest = int32_t(task_dest.size());
    // dense diagonal blocks: column-side units of kDenseCols columns of one
    // block part of a row tile (width 0), each with its own row-sum slice
    int32_t n_dslices = 0;
    for (size_t ti = 0; ti < tiles.size(); ++ti) {
        RowTile& R = tiles[ti];
        R.ds0 = n_dslices;
        for (int32_t j = 0; j < R.ndense; ++j) {
            const TileDense& D = tdense[size_t(R.dense0 + j)];
            for (int32_t k0 = 0; k0 < D.cols; k0 += kDenseCols) {
                ColTask T{};
                T.col0 = R.dense0 + j;
                T.chunk0 = k0;
                T.n = std::min(kDenseCols, D.cols - k0);
                T.stride = int32_t(ti);
                T.comp_idx = n_dslices++;
                T.nparts = 1;
                T.split_id = -1;
                T.cps = 1;
                tasks.push_back(T);
            }
        }
        R.nds = n_dslices - R.ds0;
    }
    L.n_dslices = n_dslices;
    L.n_tasks = int32_t(tasks.size());
    L.n_units = int32_t(unit_list.size());
    L.n_slots = int32_t(n_slots);
    L.n_tdense = int32_t(tdense.size());
    L.stored_p_bytes = pcodes.size();
    if (qcodes.size() >= (1ull << 42) || pcodes.size() >= (1ull << 42))
        throw overflow_error("packed factors too large for the device layout");

    // ---- arena sections, each 256-byte aligned.
    Sections& S = L.sec;
    size_t off = 0;
    auto place = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + std::max<size_t>(bytes, 1), 256);
        return o;
    };
    const size_t C = m.width.size();
    S.perm = place(4 * m.order);
    S.iperm = place(4 * m.order);  // source index -> clustered position
    S.lr = place(sizeof(LowRankDesc) * lr.size());
    S.dd = place(sizeof(DenseDesc) * dd.size());
    S.comp_w = place(C);
    S.comp_s = place(8 * C);
    S.tasks = place(sizeof(ColTask) * tasks.size());
    S.task_rec = place(sizeof(TaskRec) * task_rec.size());
    S.qcodes = place(qcodes.size() + 16);
    S.pcodes = place(pcodes.size() + 16);
    S.dense = place(8 * dense_cm.size());
    S.tiles = place(sizeof(RowTile) * tiles.size());
    S.tdense = place(sizeof(TileDense) * tdense.size());
    S.units = place(sizeof(RowUnit) * unit_list.size());
    S.kp_info = place(kp_info.size() + 16);
    S.slot_rec = place(sizeof(SlotRec) * slot_rec.size());
    S.task_dest = place(sizeof(TaskDest) * task_dest.size());
    S.row_steps = place(4 * row_steps.size());
    S.comp_sl = place(8 * C);
    S.comp_sr = place(8 * C);
    S.total = off;

    L.arena.assign(S.total, 0);
    auto& A = L.arena;
    for (uint64_t i = 0; i < m.order; ++i) {
        at<int32_t>(A, S.perm)[i] = int32_t(m.permutation[i]);
        at<int32_t>(A, S.iperm)[m.permutation[i]] = int32_t(i);
    }
    if (!lr.empty()) std::memcpy(at<LowRankDesc>(A, S.lr), lr.data(), sizeof(LowRankDesc) * lr.size());
    if (!dd.empty()) std::memcpy(at<DenseDesc>(A, S.dd), dd.data(), sizeof(DenseDesc) * dd.size());
    for (size_t c = 0; c < C; ++c) {
        at<uint8_t>(A, S.comp_w)[c] = m.width[c];
        // One rounding: s_P * s_Q.  In exact arithmetic the block contribution
        // sum_j (s_P c_P)(sum_k s_Q c_Q x) equals sum_j c_P (s_P s_Q) sum_k c_Q x.
        at<double>(A, S.comp_s)[c] = m.left_scale[c] * m.right_scale[c];
        at<double>(A, S.comp_sl)[c] = m.left_scale[c];
        at<double>(A, S.comp_sr)[c] = m.right_scale[c];
    }
    if (!tasks.empty()) std::memcpy(at<ColTask>(A, S.tasks), tasks.data(), sizeof(ColTask) * tasks.size());
    if (!task_rec.empty()) std::memcpy(A.data() + S.task_rec, task_rec.data(), sizeof(TaskRec) * task_rec.size());
    if (!qcodes.empty()) std::memcpy(A.data() + S.qcodes, qcodes.data(), qcodes.size());
    if (!pcodes.empty()) std::memcpy(A.data() + S.pcodes, pcodes.data(), pcodes.size());
    if (!kp_info.empty()) std::memcpy(A.data() + S.kp_info, kp_info.data(), kp_info.size());
    if (!unit_list.empty()) std::memcpy(A.data() + S.units, unit_list.data(), sizeof(RowUnit) * unit_list.size());
    if (!slot_rec.empty()) std::memcpy(A.data() + S.slot_rec, slot_rec.data(), sizeof(SlotRec) * slot_rec.size());
    if (!task_dest.empty()) std::memcpy(A.data() + S.task_dest, task_dest.data(), sizeof(TaskDest) * task_dest.size());
    if (!row_steps.empty()) std::memcpy(A.data() + S.row_steps, row_steps.data(), 4 * row_steps.size());
    if (!dense_cm.empty()) std::memcpy(A.data() + S.dense, dense_cm.data(), 8 * dense_cm.size());
    if (!tiles.empty()) std::memcpy(A.data() + S.tiles, tiles.data(), sizeof(RowTile) * tiles.size());
    if (!tdense.empty()) std::memcpy(A.data() + S.tdense, tdense.data(), sizeof(TileDense) * tdense.size());
    return L;
}

}  // namespace qhg

extern "C" uint64_t qh_fnv1a64(const void* bytes, size_t len) {
    const auto* p = static_cast<const uint8_t*>(bytes);
    uint64_t h = qhg::kFnvOffsetBasis;
    for (size_t i = 0; i < len; ++i) h = (h ^ p[i]) * qhg::kFnvPrimeValue;
    return h;
}
