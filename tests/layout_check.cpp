// CPU check of the resident layout (test infrastructure, built by
// tests/test_layout.py with the library's layout.cpp): for a QHMAT001 file,
// decode every stored digit plane back into codes and compare them with the
// file's codes (the reference's decode, src/qhmat/core.cpp:269-282), and
// check the work lists the kernels rely on.  Prints "OK ..." and exits 0, or
// prints the first mismatches and exits 1.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <set>
#include <vector>

#include "layout.hpp"

using namespace qhg;

namespace {

int fails = 0;
#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            if (fails < 20) {                     \
                std::printf("FAIL: " __VA_ARGS__); \
                std::printf("\n");                \
            }                                     \
            ++fails;                              \
        }                                         \
    } while (0)

// The reference's decode of code i of a run of width w (sign-extended).
int64_t ref_code(const uint32_t* run, uint64_t i, int w) {
    const uint64_t pos = i * uint64_t(w), wi = pos >> 5, off = pos & 31;
    uint64_t v = run[wi];
    if (off + uint64_t(w) > 32) v |= uint64_t(run[wi + 1]) << 32;
    const uint64_t f = (v >> off) & ((uint64_t(1) << w) - 1);
    return (f >> (w - 1)) ? int64_t(f) - (int64_t(1) << w) : int64_t(f);
}

// Digit of (k-block kb, entry e) in a group row (the inverse of the writer's
// fragment order: thread t = (e & 7) >> 1 holds entries 2t, 2t+1, 2t+8, 2t+9).
uint32_t get_digit(const uint8_t* row, bool nib, int kb, int e) {
    const int t = (e & 7) >> 1, slot = (e & 1) | ((e >> 3) << 1);
    if (!nib) return row[8 * t + 4 * kb + slot];
    uint32_t w;
    std::memcpy(&w, row + 4 * t, 4);
    const int nibble = 2 * kb + (slot >> 1) + 4 * (slot & 1);
    return (w >> (4 * nibble)) & 15u;
}

// A code from its planes: lower digits unsigned, the top one offset by
// 2^(tb-1).
int64_t from_digits(const std::vector<uint32_t>& d, int tb) {
    int64_t c = 0;
    const int P = int(d.size());
    for (int m = 0; m < P - 1; ++m) c += int64_t(d[size_t(m)]) << (8 * m);
    c += (int64_t(d[size_t(P - 1)]) - (int64_t(1) << (tb - 1))) * (int64_t(1) << (8 * (P - 1)));
    return c;
}

template <class T>
const T* sec(const Layout& L, size_t off) {
    return reinterpret_cast<const T*>(L.arena.data() + off);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::ifstream f(argv[1], std::ios::binary);
    std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), {});
    const HostMatrix m = parse_qhmat(bytes.data(), bytes.size());
    const Layout L = build_layout(m);
    const auto* tasks = sec<ColTask>(L, L.sec.tasks);
    const auto* trec = sec<TaskRec>(L, L.sec.task_rec);
    const auto* tdest = sec<TaskDest>(L, L.sec.task_dest);
    const uint8_t* qcodes = sec<uint8_t>(L, L.sec.qcodes);
    const uint8_t* pcodes = sec<uint8_t>(L, L.sec.pcodes);
    const auto* tiles = sec<RowTile>(L, L.sec.tiles);
    const auto* tdense = sec<TileDense>(L, L.sec.tdense);
    const auto* units = sec<RowUnit>(L, L.sec.units);
    const uint8_t* kpi = sec<uint8_t>(L, L.sec.kp_info);
    const auto* srec = sec<SlotRec>(L, L.sec.slot_rec);
    const auto* steps = sec<uint32_t>(L, L.sec.row_steps);

    // component -> its block's row0 (left factor rows start there)
    std::vector<uint64_t> comp_row0(m.width.size(), 0);
    for (const auto& b : m.blocks)
        if (!b.dense)
            for (uint64_t j = 0; j < b.rank; ++j) comp_row0[b.comp0 + j] = b.row0;

    // ---- column side: every code of every component, from the digit planes
    std::vector<int> comp_seen(m.width.size(), 0);
    long long col_codes = 0;
    std::vector<int> dslice_seen(size_t(L.n_dslices), 0);
    for (int i = 0; i < L.n_tasks; ++i) {
        const ColTask& T = tasks[i];
        if (T.width == 0) {  // dense unit: columns of one block part, one slice
            CHECK(T.comp_idx >= 0 && T.comp_idx < L.n_dslices, "dense unit %d slice", i);
            if (T.comp_idx >= 0 && T.comp_idx < L.n_dslices) ++dslice_seen[size_t(T.comp_idx)];
            const RowTile& R = tiles[T.stride];
            CHECK(T.col0 >= R.dense0 && T.col0 < R.dense0 + R.ndense, "dense unit %d block part", i);
            CHECK(T.comp_idx >= R.ds0 && T.comp_idx < R.ds0 + R.nds, "dense unit %d slice of its tile", i);
            CHECK(T.n > 0 && T.n <= kDenseCols && T.chunk0 + T.n <= tdense[T.col0].cols, "dense unit %d columns", i);
            continue;
        }
        const int w = T.width, P = code_planes(w), tb = w - 8 * (P - 1);
        const bool nibtop = top_is_nibble(w);
        const int row_bytes = (P - 1) * 32 + (nibtop ? 16 : 32);
        CHECK(T.stride == T.count * row_bytes, "task %d stride", i);
        for (int l = 0; l < T.count; ++l) {
            const int32_t c = trec[T.comp_idx + l].comp;
            CHECK(trec[T.comp_idx + l].width == w, "task %d row %d width", i, l);
            if (T.part == 0) ++comp_seen[size_t(c)];
            const uint32_t* run = m.right_words.data() + m.right_off[size_t(c)];
            const int q = l / 16, r = l % 16, rows_q = std::min(16, T.count - 16 * q);
            for (int ch = T.chunk0; ch < T.chunk0 + T.nchunks; ++ch) {
                size_t goff = size_t(T.off) + size_t(ch) * size_t(T.stride) + size_t(q) * 16 * size_t(row_bytes);
                std::vector<const uint8_t*> rows;
                for (int mm = 0; mm < P; ++mm) {
                    const bool nb = nibtop && mm == P - 1;
                    rows.push_back(qcodes + goff + size_t(r) * (nb ? 16 : 32));
                    goff += size_t(rows_q) * (nb ? 16 : 32);
                }
                for (int e = 0; e < kColChunk; ++e) {
                    const int64_t idx = int64_t(ch) * kColChunk + e;
                    std::vector<uint32_t> d;
                    for (int mm = 0; mm < P; ++mm) d.push_back(get_digit(rows[size_t(mm)], nibtop && mm == P - 1, e >> 4, e & 15));
                    const int64_t want = idx < T.n ? ref_code(run, uint64_t(idx), w) : 0;
                    CHECK(from_digits(d, tb) == want, "column code: task %d comp %d entry %lld", i, c, (long long)idx);
                    if (idx < T.n) ++col_codes;
                }
            }
        }
    }
    for (size_t c = 0; c < m.width.size(); ++c) CHECK(comp_seen[c] == 1, "component %zu in %d column tasks", c, comp_seen[c]);
    for (int s = 0; s < L.n_dslices; ++s) CHECK(dslice_seen[size_t(s)] == 1, "dense slice %d", s);

    // ---- row side: every code from the units' digit groups; slots; steps
    long long row_codes = 0;
    for (int u = 0; u < L.n_units; ++u) {
        const RowUnit& U = units[u];
        const RowTile& R = tiles[U.tile];
        const uint8_t* gp = pcodes + U.code_off;
        int kstep = 0;
        for (int s = 0; s < U.nsteps; ++s) {
            const uint32_t sw = steps[U.step0 + s];
            const int c = int(sw & 255u);
            if (sw >> 24) {
                for (int k = kstep; k < kstep + c; ++k) {
                    const int kp = U.h + k * U.H;
                    CHECK(kpi[U.kp_off + kp] == ((sw >> 16) & 255u), "unit %d step %d uniform info", u, s);
                    CHECK(32 * (kp + 1) <= U.K, "unit %d step %d uniform inside the k axis", u, s);
                }
            }
            kstep += c;
        }
        CHECK(kstep == U.nkps, "unit %d steps cover %d of %d k-pairs", u, kstep, U.nkps);
        for (int i = 0; i < U.nkps; ++i) {
            const int kp = U.h + i * U.H;
            const int info = kpi[U.kp_off + kp];
            const int planes = info & 7, tb = (info >> 4) + 1;
            const bool nib = (info >> 3) & 1;
            std::vector<const uint8_t*> grp;
            for (int mm = 0; mm < planes; ++mm) {
                grp.push_back(gp);
                gp += (nib && mm == planes - 1) ? 256 : 512;
            }
            for (int e = 0; e < 32; ++e) {
                const int k = 32 * kp + e;
                if (k >= U.K) break;
                const SlotRec sr = srec[U.slot0 + 32 * i + e];
                CHECK(sr.comp >= 0, "unit %d slot of k %d has no component", u, k);
                if (sr.comp < 0) continue;
                const int w = sr.info & 255;
                CHECK(w == m.width[size_t(sr.comp)], "slot width");
                const uint32_t* run = m.left_words.data() + m.left_off[size_t(sr.comp)];
                for (int rr = 0; rr < 16; ++rr) {
                    const int tr = 16 * U.q + rr;
                    if (tr >= R.rows) break;
                    std::vector<uint32_t> d;
                    for (int mm = 0; mm < planes; ++mm) {
                        const bool nb = nib && mm == planes - 1;
                        d.push_back(get_digit(grp[size_t(mm)] + size_t(rr) * (nb ? 16 : 32), nb, e >> 4, e & 15));
                    }
                    const uint64_t br = uint64_t(R.row0 + tr) - comp_row0[size_t(sr.comp)];
                    CHECK(from_digits(d, tb) == ref_code(run, br, w), "row code: unit %d k %d row %d", u, k, tr);
                    ++row_codes;
                }
            }
        }
    }

    // ---- B rows: every slot with a component is written by exactly one
    // destination record, of a task holding that component
    std::vector<int> fed(size_t(L.n_slots), 0);
    for (int i = 0; i < L.n_tasks; ++i) {
        const ColTask& T = tasks[i];
        if (T.width == 0 || (T.nparts > 1 && T.part != 0)) continue;
        for (int d = 0; d < T.ndest; ++d) {
            const TaskDest D = tdest[T.dest0 + d];
            const int row = (D.row_cexp >> 16) & 31;
            CHECK(row < T.count, "task %d dest row", i);
            CHECK(D.slot >= 0 && D.slot < L.n_slots, "task %d dest slot", i);
            if (D.slot < 0 || D.slot >= L.n_slots) continue;
            ++fed[size_t(D.slot)];
            CHECK(srec[D.slot].comp == trec[T.comp_idx + row].comp, "task %d dest %d component", i, d);
        }
    }
    long long slots_used = 0;
    for (int s = 0; s < L.n_slots; ++s) {
        if (srec[s].comp >= 0) {
            CHECK(fed[size_t(s)] == 1, "slot %d written %d times", s, fed[size_t(s)]);
            ++slots_used;
        } else {
            CHECK(fed[size_t(s)] == 0, "padding slot %d written", s);
        }
    }
    if (fails) {
        std::printf("%d failures\n", fails);
        return 1;
    }
    std::printf("OK column codes %lld row codes %lld slots %lld tasks %d units %d dense slices %d\n", col_codes,
                row_codes, slots_used, L.n_tasks, L.n_units, L.n_dslices);
    return 0;
}
