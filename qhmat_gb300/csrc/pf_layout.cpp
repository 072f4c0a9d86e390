// Construction of the precision form's resident layout (see pf_layout.hpp).
#include "pf_layout.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <utility>

namespace qhg {
namespace {

// Code i of a run of width w (LSB-first bit string, sign-extended): the field
// HMatrix::decode reads (src/qhmat/core.cpp:269-282).
int32_t pf_code(const uint32_t* run, uint64_t i, int w) {
    const uint64_t pos = i * uint64_t(w), wi = pos >> 5, off = pos & 31;
    uint64_t v = run[wi];
    if (off + uint64_t(w) > 32) v |= uint64_t(run[wi + 1]) << 32;
    const uint64_t f = (v >> off) & ((uint64_t(1) << w) - 1);
    return int32_t(int64_t(f << (64 - w)) >> (64 - w));
}

int planes_of(int w) { return (w + 7) / 8; }

// Digit byte m of a code on P planes: unsigned lower digits, signed top digit.
uint8_t digit(int32_t c, int m, int P) {
    if (m < P - 1) return uint8_t((c >> (8 * m)) & 255);
    return uint8_t(int8_t(c >> (8 * (P - 1))));
}

// IEEE binary16 bits of v, rounded to nearest even (|v| < 65520; subnormals
// kept).
uint16_t f16_bits(double v) {
    const uint16_t sign = std::signbit(v) ? 0x8000 : 0;
    double a = std::fabs(v);
    if (a == 0.0) return sign;
    int e;
    std::frexp(a, &e);  // a = f 2^e, f in [0.5, 1)
    int E = e - 1;      // a in [2^E, 2^(E+1))
    if (E < -14) E = -14;  // subnormal range: fixed quantum 2^-24
    const double q = std::ldexp(1.0, E - 10);
    double mant = std::nearbyint(a / q);  // round to nearest even (default mode)
    if (mant >= 2048.0) {  // rounded up to the next binade
        mant /= 2.0;
        ++E;
    }
    if (E > 15) throw std::overflow_error("f16 limb out of range");
    if (mant < 1024.0) return uint16_t(sign | uint16_t(mant));  // subnormal
    return uint16_t(sign | uint16_t((E + 15) << 10) | (uint16_t(mant) & 0x3FF));
}

double f16_value(uint16_t h) {
    const int e = (h >> 10) & 31, f = h & 0x3FF;
    const double m = e == 0 ? std::ldexp(double(f), -24) : std::ldexp(double(1024 + f), e - 25);
    return (h & 0x8000) ? -m : m;
}

// Byte offset of element (r, c) of a 128 x 64 f16 operand tile in the
// 128-byte-swizzled K-major layout: 8-row groups of 1024 bytes, 16-byte chunk
// index c/8 XOR-ed with r mod 8.
size_t swz(int r, int c) {
    return size_t(r / 8) * 1024 + size_t(r % 8) * 128 + size_t(((c / 8) ^ (r % 8)) * 16) + size_t(c % 8) * 2;
}

// Longest-processing-time assignment of items (cost) to W workers; returns
// the item order (worker-major) and W + 1 offsets.
void lpt(const std::vector<double>& cost, int W, std::vector<int32_t>& order, std::vector<int32_t>& off) {
    const int n = int(cost.size());
    std::vector<int32_t> idx(static_cast<size_t>(n));
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return cost[size_t(a)] > cost[size_t(b)]; });
    using Load = std::pair<double, int32_t>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int32_t w = 0; w < W; ++w) heap.push({0.0, w});
    std::vector<std::vector<int32_t>> lists(static_cast<size_t>(W));
    for (int32_t i : idx) {
        Load l = heap.top();
        heap.pop();
        lists[size_t(l.second)].push_back(i);
        l.first += cost[size_t(i)];
        heap.push(l);
    }
    order.clear();
    off.assign(size_t(W) + 1, 0);
    for (int32_t w = 0; w < W; ++w) {
        off[size_t(w)] = int32_t(order.size());
        order.insert(order.end(), lists[size_t(w)].begin(), lists[size_t(w)].end());
    }
    off[size_t(W)] = int32_t(order.size());
}

size_t align_to(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

PfLayout build_pf_layout(const HostMatrix& m, int grid, double row_items_per_cta) {
    PfLayout L;
    L.order = m.order;
    L.bound = m.reconstruction_bound();
    L.grid = std::max(1, grid);
    if (m.order >= (1ull << 30)) throw std::overflow_error("matrix order too large for the precision layout");
    const int64_t n = int64_t(m.order);

    // components of the low-rank blocks
    struct Comp {
        int32_t block, j, w, P;
    };
    std::vector<Comp> comps;
    for (size_t k = 0; k < m.blocks.size(); ++k) {
        const auto& b = m.blocks[k];
        if (b.dense) {
            L.dense_bytes += 8ull * (b.row1 - b.row0) * (b.col1 - b.col0);
            continue;
        }
        for (uint64_t j = 0; j < b.rank; ++j) {
            const int w = m.width[size_t(b.comp0 + j)];
            comps.push_back({int32_t(k), int32_t(j), w, planes_of(w)});
            L.code_bytes += 4ull * (words_for_bits(b.row1 - b.row0, w) + words_for_bits(b.col1 - b.col0, w));
            L.scale_bytes += 16;
        }
    }
    L.n_comp = int32_t(comps.size());
    auto gcomp = [&](const Comp& c) { return size_t(m.blocks[size_t(c.block)].comp0) + size_t(c.j); };

    // ---- row side: 128-row tiles; K axis = components of blocks meeting the tile
    const int32_t n_tiles = int32_t((n + kPfM - 1) / kPfM);
    L.n_tiles = n_tiles;
    std::vector<std::vector<std::pair<int32_t, int32_t>>> tile_slots(static_cast<size_t>(n_tiles));  // (comp index, half)
    std::vector<std::vector<int32_t>> tile_dense(static_cast<size_t>(n_tiles));
    {
        // blocks per tile
        std::vector<std::vector<int32_t>> by_block(m.blocks.size());
        for (size_t ci = 0; ci < comps.size(); ++ci) by_block[size_t(comps[ci].block)].push_back(int32_t(ci));
        for (size_t k = 0; k < m.blocks.size(); ++k) {
            const auto& b = m.blocks[k];
            if (b.row1 == b.row0 || b.col1 == b.col0) continue;
            const int64_t t0 = int64_t(b.row0) / kPfM, t1 = (int64_t(b.row1) - 1) / kPfM;
            for (int64_t t = t0; t <= t1; ++t) {
                if (b.dense) {
                    tile_dense[size_t(t)].push_back(int32_t(k));
                    continue;
                }
                const int64_t r0 = std::max<int64_t>(int64_t(b.row0), t * kPfM) - t * kPfM;
                const int64_t r1 = std::min<int64_t>(int64_t(b.row1), (t + 1) * kPfM) - t * kPfM;
                const int half = r1 <= 64 ? 1 : (r0 >= 64 ? 2 : 0);
                for (int32_t ci : by_block[k]) tile_slots[size_t(t)].push_back({ci, half});
            }
        }
    }

    std::vector<PfRowChunk> chunks;
    std::vector<std::vector<int32_t>> comp_dests(comps.size());
    std::vector<uint8_t> praw;
    std::vector<double> tile_cost(static_cast<size_t>(n_tiles), 0.0);
    std::vector<int32_t> tile_chunk0(size_t(n_tiles) + 1, 0), tile_dexp(static_cast<size_t>(n_tiles), 0);
    int32_t slot_base = 0;
    for (int32_t t = 0; t < n_tiles; ++t) {
        if (slot_base >= (1 << 28) - 2 * kPfK) throw std::overflow_error("too many row-side slots for the precision layout");
        tile_chunk0[size_t(t)] = int32_t(chunks.size());
        auto& sl = tile_slots[size_t(t)];
        // halves 1, 2, then full; widest first inside each
        std::stable_sort(sl.begin(), sl.end(), [&](const auto& a, const auto& b) {
            const int ha = a.second == 0 ? 3 : a.second, hb = b.second == 0 ? 3 : b.second;
            if (ha != hb) return ha < hb;
            return comps[size_t(a.first)].w > comps[size_t(b.first)].w;
        });
        const int64_t trow0 = int64_t(t) * kPfM;
        size_t i = 0;
        while (i < sl.size()) {
            const int half = sl[i].second;
            size_t j = i;
            while (j < sl.size() && sl[j].second == half && j - i < size_t(kPfK)) ++j;
            const int nvalid = int(j - i);
            const int P = comps[size_t(sl[i].first)].P;  // widest first
            const int stored_rows = half == 0 ? 128 : 64;
            const int row_off = half == 2 ? 64 : 0;
            PfRowChunk ch{};
            ch.a_off = int64_t(praw.size());
            ch.b = slot_base;
            ch.kind = 0;
            ch.planes = uint8_t(P);
            ch.half = uint8_t(half);
            ch.nvalid = uint8_t(nvalid);
            praw.resize(praw.size() + size_t(P) * size_t(stored_rows) * kPfK, 0);
            uint8_t* base = praw.data() + ch.a_off;
            for (int k = 0; k < nvalid; ++k) {
                const Comp& c = comps[size_t(sl[i + size_t(k)].first)];
                const auto& b = m.blocks[size_t(c.block)];
                const size_t g = gcomp(c);
                const uint32_t* run = m.left_words.data() + m.left_off[g];
                comp_dests[size_t(sl[i + size_t(k)].first)].push_back(slot_base + k | (P - 1) << 28);
                for (int r = 0; r < stored_rows; ++r) {
                    const int64_t R = trow0 + row_off + r;
                    if (R < int64_t(b.row0) || R >= int64_t(b.row1)) continue;
                    const int32_t code = pf_code(run, uint64_t(R - int64_t(b.row0)), c.w);
                    for (int mm = 0; mm < P; ++mm)
                        base[size_t(mm) * size_t(stored_rows) * kPfK + size_t(r) * kPfK + size_t(k)] = digit(code, mm, P);
                }
            }
            L.stored_p += size_t(P) * size_t(stored_rows) * kPfK;
            L.mma_row += uint64_t(P) * kPfM * kPfK;
            tile_cost[size_t(t)] += 4.0 * P + 3.0;
            chunks.push_back(ch);
            slot_base += kPfK;
            i = j;
        }
        // dense blocks meeting the tile: 64-column parts as three f16 limb tiles
        double dmax = 0.0;
        for (int32_t k : tile_dense[size_t(t)]) {
            const auto& b = m.blocks[size_t(k)];
            const uint64_t nn = b.col1 - b.col0;
            for (uint64_t R = std::max<uint64_t>(b.row0, uint64_t(trow0));
                 R < std::min<uint64_t>(b.row1, uint64_t(trow0 + kPfM)); ++R)
                for (uint64_t cc = 0; cc < nn; ++cc)
                    dmax = std::max(dmax, std::fabs(m.dense[b.dense_off + (R - b.row0) * nn + cc]));
        }
        const int dexp = dmax > 0.0 ? std::ilogb(dmax) + 1 - 15 : 0;  // max |D| 2^-dexp < 2^15
        tile_dexp[size_t(t)] = dexp;
        for (int32_t k : tile_dense[size_t(t)]) {
            const auto& b = m.blocks[size_t(k)];
            const int64_t nn = int64_t(b.col1 - b.col0);
            const int64_t e_base = int64_t(b.col0) & ~int64_t(7);
            const int64_t shift = int64_t(b.col0) - e_base;
            const int64_t nch = (shift + nn + kPfK - 1) / kPfK;
            for (int64_t c = 0; c < nch; ++c) {
                PfRowChunk ch{};
                ch.a_off = int64_t(praw.size());
                ch.b = int32_t(e_base + c * kPfK);
                ch.kind = 1;
                ch.planes = 3;
                ch.half = 0;
                ch.nvalid = kPfK;
                praw.resize(praw.size() + 3 * size_t(kPfTileBytes), 0);
                uint8_t* base = praw.data() + ch.a_off;
                for (int r = 0; r < kPfM; ++r) {
                    const int64_t R = trow0 + r;
                    if (R < int64_t(b.row0) || R >= int64_t(b.row1)) continue;
                    for (int col = 0; col < kPfK; ++col) {
                        const int64_t e = e_base + c * kPfK + col;
                        if (e < int64_t(b.col0) || e >= int64_t(b.col1)) continue;
                        const double v = std::ldexp(m.dense[b.dense_off + uint64_t(R - int64_t(b.row0)) * uint64_t(nn) +
                                                            uint64_t(e - int64_t(b.col0))],
                                                    -dexp);
                        const uint16_t h0 = f16_bits(v);
                        const double r1 = v - f16_value(h0);
                        const uint16_t h1 = f16_bits(r1);
                        const double r2 = r1 - f16_value(h1);
                        const uint16_t h2 = f16_bits(r2);
                        const uint16_t hs[3] = {h0, h1, h2};
                        for (int l = 0; l < 3; ++l)
                            std::memcpy(base + size_t(l) * kPfTileBytes + swz(r, col), &hs[l], 2);
                    }
                }
                L.stored_dense += 3 * size_t(kPfTileBytes);
                L.mma_row += 3ull * kPfM * kPfK;
                tile_cost[size_t(t)] += 12.0 + 6.0;
                chunks.push_back(ch);
            }
        }
    }
    tile_chunk0[size_t(n_tiles)] = int32_t(chunks.size());
    L.n_slots = slot_base;
    L.n_chunks = int32_t(chunks.size());
    if (int64_t(praw.size()) >= (int64_t(1) << 40)) throw std::overflow_error("precision layout too large");

    // row items: each tile's chunk list cut into K splits of about equal cost
    std::vector<PfRowItem> row_items;
    std::vector<double> row_cost;
    {
        const double total = std::accumulate(tile_cost.begin(), tile_cost.end(), 0.0);
        const double per_cta = row_items_per_cta > 0.0 ? std::max(1.0, row_items_per_cta) : 3.0;
        const double target = std::max(1.0, total / (per_cta * L.grid));
        L.tile_part0.assign(size_t(n_tiles) + 1, 0);
        int32_t part = 0;
        for (int32_t t = 0; t < n_tiles; ++t) {
            L.tile_part0[size_t(t)] = part;
            const int32_t c0 = tile_chunk0[size_t(t)], c1 = tile_chunk0[size_t(t) + 1];
            const int H = std::max(1, std::min<int>(c1 - c0, int(std::ceil(tile_cost[size_t(t)] / target))));
            auto cost_of = [&](int32_t c) { return chunks[size_t(c)].kind ? 18.0 : 4.0 * chunks[size_t(c)].planes + 3.0; };
            int32_t c = c0;
            double acc = 0.0;
            for (int h = 0; h < H; ++h) {
                const double want = tile_cost[size_t(t)] * (h + 1) / H;
                const int32_t start = c;
                while (c < c1 && (h == H - 1 || c == start || acc + 0.5 * cost_of(c) <= want)) acc += cost_of(c++);
                PfRowItem it{};
                it.tile = t;
                it.row0 = int32_t(int64_t(t) * kPfM);
                it.rows = int32_t(std::min<int64_t>(kPfM, n - int64_t(t) * kPfM));
                it.part = part++;
                it.chunk0 = start;
                it.nchunks = c - start;
                it.dense_exp = tile_dexp[size_t(t)];
                double ic = 20.0;  // epilogue
                for (int32_t q = start; q < c; ++q) ic += cost_of(q);
                row_items.push_back(it);
                row_cost.push_back(ic);
            }
        }
        L.tile_part0[size_t(n_tiles)] = part;
        L.n_parts = part;
    }
    // the row item holding each low-rank slot (for the items' own u bounds)
    std::vector<int32_t> item_of_slot(size_t(L.n_slots), -1);
    for (size_t i = 0; i < row_items.size(); ++i)
        for (int32_t c = row_items[i].chunk0; c < row_items[i].chunk0 + row_items[i].nchunks; ++c)
            if (chunks[size_t(c)].kind == 0)
                for (int32_t sl = chunks[size_t(c)].b; sl < chunks[size_t(c)].b + kPfK && sl < L.n_slots; ++sl)
                    item_of_slot[size_t(sl)] = int32_t(i);
    std::vector<double> item_ubound(row_items.size(), 0.0);

    // ---- column side: components grouped by column range, widest first, 128 per item
    std::map<std::pair<uint64_t, uint64_t>, std::vector<int32_t>> groups;
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        const auto& b = m.blocks[size_t(comps[ci].block)];
        if (b.col1 > b.col0 && b.row1 > b.row0) groups[{b.col0, b.col1 - b.col0}].push_back(int32_t(ci));
    }
    std::vector<PfColItem> col_items;
    std::vector<double> col_cost;
    std::vector<PfComp> pcomps;
    std::vector<int32_t> dests;
    std::vector<uint8_t> qraw;
    double ubound = 0.0;
    for (auto& kv : groups) {
        const int64_t col0 = int64_t(kv.first.first), nn = int64_t(kv.first.second);
        auto& list = kv.second;
        std::stable_sort(list.begin(), list.end(), [&](int32_t a, int32_t b) { return comps[size_t(a)].w > comps[size_t(b)].w; });
        const int64_t e_base = col0 & ~int64_t(7), shift = col0 - e_base;
        const int32_t nkc = int32_t((shift + nn + kPfK - 1) / kPfK);
        for (size_t i0 = 0; i0 < list.size(); i0 += kPfM) {
            const int count = int(std::min<size_t>(kPfM, list.size() - i0));
            const int P = comps[size_t(list[i0])].P;
            PfColItem it{};
            it.a_off = int64_t(qraw.size());
            it.e_base = int32_t(e_base);
            it.nkc = nkc;
            it.planes = P;
            it.count = count;
            it.comp0 = int32_t(pcomps.size());
            qraw.resize(qraw.size() + size_t(nkc) * size_t(P) * kPfPlaneBytes, 0);
            uint8_t* base = qraw.data() + it.a_off;
            for (int j = 0; j < count; ++j) {
                const int32_t ci = list[i0 + size_t(j)];
                const Comp& c = comps[size_t(ci)];
                const size_t g = gcomp(c);
                const uint32_t* run = m.right_words.data() + m.right_off[g];
                double l1 = 0.0;  // ||c^Q_j||_1
                for (int64_t e = 0; e < nn; ++e) {
                    const int32_t code = pf_code(run, uint64_t(e), c.w);
                    l1 += std::fabs(double(code));
                    const int64_t col = shift + e, kc = col / kPfK, cc = col % kPfK;
                    for (int mm = 0; mm < P; ++mm)
                        base[(size_t(kc) * size_t(P) + size_t(mm)) * kPfPlaneBytes + size_t(j) * kPfK + size_t(cc)] =
                            digit(code, mm, P);
                }
                PfComp pc{};
                pc.scale = m.left_scale[g] * m.right_scale[g];
                // |u_j| <= |s^P s^Q| ||c^Q_j||_1 max|x|; the row side scales u by
                // 256^(P-1) of its chunk: track the largest such bound
                // (overall, and per row item over the slots it holds)
                const double ub0 = std::fabs(pc.scale) * l1;
                for (int32_t dw : comp_dests[size_t(ci)]) {
                    const double ub = ub0 * std::ldexp(1.0, 8 * (dw >> 28));
                    if (!(ub > 0.0 && std::isfinite(ub))) continue;
                    ubound = std::max(ubound, ub);
                    const int32_t item = item_of_slot[size_t(dw & 0x0FFFFFFF)];
                    if (item >= 0) item_ubound[size_t(item)] = std::max(item_ubound[size_t(item)], ub);
                }
                pc.dest0 = int32_t(dests.size());
                pc.ndest = int32_t(comp_dests[size_t(ci)].size());
                dests.insert(dests.end(), comp_dests[size_t(ci)].begin(), comp_dests[size_t(ci)].end());
                pcomps.push_back(pc);
            }
            L.stored_q += size_t(nkc) * size_t(P) * kPfPlaneBytes;
            L.mma_col += uint64_t(nkc) * uint64_t(P) * kPfM * kPfK;
            col_items.push_back(it);
            col_cost.push_back(double(nkc) * (4.0 * P + 3.0) + 10.0);
        }
    }
    if (int64_t(qraw.size()) >= (int64_t(1) << 40)) throw std::overflow_error("precision layout too large");
    // 2^u_beta > every |u_j| 256^(P-1) / max|x| (with a factor 2 of room for
    // the FP32 rounding of u)
    L.u_beta = ubound > 0.0 ? std::ilogb(ubound) + 2 : 0;
    for (size_t i = 0; i < row_items.size(); ++i)
        row_items[i].u_beta = item_ubound[i] > 0.0 ? std::ilogb(item_ubound[i]) + 2 : L.u_beta;
    L.n_col_items = int32_t(col_items.size());
    L.n_row_items = int32_t(row_items.size());
    L.n_dests = int32_t(dests.size());

    // static schedules: items in CTA-major order, longest first per CTA
    std::vector<int32_t> corder, coff, rorder, roff;
    lpt(col_cost, L.grid, corder, coff);
    lpt(row_cost, L.grid, rorder, roff);
    {
        std::vector<PfColItem> tmp(col_items);
        for (size_t i = 0; i < corder.size(); ++i) col_items[i] = tmp[size_t(corder[i])];
        std::vector<PfRowItem> tmp2(row_items);
        for (size_t i = 0; i < rorder.size(); ++i) row_items[i] = tmp2[size_t(rorder[i])];
    }

    // ---- arena
    PfSections& S = L.sec;
    size_t off = 0;
    auto take = [&](size_t bytes, size_t align) {
        off = align_to(off, align);
        const size_t o = off;
        off += std::max<size_t>(bytes, 16);
        return o;
    };
    S.perm = take(4 * size_t(n), 128);
    S.col_items = take(sizeof(PfColItem) * col_items.size(), 128);
    S.comps = take(sizeof(PfComp) * pcomps.size(), 128);
    S.dests = take(4 * dests.size(), 128);
    S.row_items = take(sizeof(PfRowItem) * row_items.size(), 128);
    S.chunks = take(sizeof(PfRowChunk) * chunks.size(), 128);
    S.col_sched = take(4 * coff.size(), 128);
    S.row_sched = take(4 * roff.size(), 128);
    S.qraw = take(qraw.size(), 1024);
    S.praw = take(praw.size(), 1024);
    S.total = align_to(off, 1024);
    L.arena.assign(S.total, 0);
    uint8_t* A = L.arena.data();
    for (int64_t i = 0; i < n; ++i) {
        const int32_t v = int32_t(m.permutation[size_t(i)]);
        std::memcpy(A + S.perm + 4 * size_t(i), &v, 4);
    }
    auto put = [&](size_t at, const void* src, size_t bytes) {
        if (bytes) std::memcpy(A + at, src, bytes);
    };
    put(S.col_items, col_items.data(), sizeof(PfColItem) * col_items.size());
    put(S.comps, pcomps.data(), sizeof(PfComp) * pcomps.size());
    put(S.dests, dests.data(), 4 * dests.size());
    put(S.row_items, row_items.data(), sizeof(PfRowItem) * row_items.size());
    put(S.chunks, chunks.data(), sizeof(PfRowChunk) * chunks.size());
    put(S.col_sched, coff.data(), 4 * coff.size());
    put(S.row_sched, roff.data(), 4 * roff.size());
    put(S.qraw, qraw.data(), qraw.size());
    put(S.praw, praw.data(), praw.size());
    return L;
}

}  // namespace qhg
