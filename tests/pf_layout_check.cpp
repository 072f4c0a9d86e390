// CPU emulation of the precision form's resident layout (test
// infrastructure, built by tests/test_pf_layout.py with the library's
// layout.cpp and pf_layout.cpp).  Reads a QHMAT001 file and a right-hand side
// (n doubles, source order), builds the precision layout, and walks the same
// work lists the GPU kernels walk -- column items (digit planes x x), the
// component -> slot destinations, row items (digit planes x u, dense limb
// tiles un-swizzled x x), the K-split partials and their combine through the
// permutation -- in exact-enough FP64 (digits recombined into the codes, dense
// limbs summed).  Writes y (source order) to the output file.  Any layout
// fault (a wrong digit, slot, row half, swizzle or split) shows as a wrong y.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <vector>

#include "layout.hpp"
#include "pf_layout.hpp"

using namespace qhg;

namespace {

template <class T>
const T* sec(const PfLayout& L, size_t off) {
    return reinterpret_cast<const T*>(L.arena.data() + off);
}

// Code from the digit bytes of planes 0..P-1 (top plane signed).
int64_t code_from(const uint8_t* plane0, size_t plane_stride, int P) {
    int64_t c = 0;
    for (int m = 0; m < P; ++m) {
        const uint8_t d = plane0[size_t(m) * plane_stride];
        const int64_t v = m == P - 1 ? int64_t(int8_t(d)) : int64_t(d);
        c += v * (int64_t(1) << (8 * m));
    }
    return c;
}

double f16_to_double(uint16_t h) {
    const int e = (h >> 10) & 31, f = h & 0x3FF;
    const double m = e == 0 ? std::ldexp(double(f), -24) : std::ldexp(double(1024 + f), e - 25);
    return (h & 0x8000) ? -m : m;
}

size_t swz(int r, int c) {
    return size_t(r / 8) * 1024 + size_t(r % 8) * 128 + size_t(((c / 8) ^ (r % 8)) * 16) + size_t(c % 8) * 2;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: pf_layout_check file.qhmat x.bin y.bin [grid]\n");
        return 2;
    }
    std::ifstream f(argv[1], std::ios::binary);
    std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    HostMatrix hm = parse_qhmat(bytes.data(), bytes.size());
    const int grid = argc > 4 ? std::atoi(argv[4]) : 7;
    PfLayout L = build_pf_layout(hm, grid);
    const int64_t n = int64_t(L.order);
    std::vector<double> xs(static_cast<size_t>(n)), y(static_cast<size_t>(n), 0.0);
    {
        std::ifstream fx(argv[2], std::ios::binary);
        fx.read(reinterpret_cast<char*>(xs.data()), std::streamsize(8 * n));
    }
    const int32_t* perm = sec<int32_t>(L, L.sec.perm);
    std::vector<double> xc(static_cast<size_t>(n) + 4096, 0.0);  // clustered order, zero past n
    for (int64_t i = 0; i < n; ++i) xc[size_t(i)] = xs[size_t(perm[i])];

    // column side: u per slot
    std::vector<double> U(size_t(L.n_slots), 0.0);
    std::vector<int> fed(size_t(L.n_slots), 0);
    std::vector<int> slot_planes;
    const auto* ci = sec<PfColItem>(L, L.sec.col_items);
    const auto* cs = sec<int32_t>(L, L.sec.col_sched);
    if (cs[0] != 0 || cs[L.grid] != L.n_col_items) {
        std::printf("FAIL column schedule offsets\n");
        return 1;
    }
    const auto* comps = sec<PfComp>(L, L.sec.comps);
    const auto* dests = sec<int32_t>(L, L.sec.dests);
    const uint8_t* qraw = L.arena.data() + L.sec.qraw;
    for (int32_t it = 0; it < L.n_col_items; ++it) {
        const PfColItem& I = ci[it];
        if (I.e_base % 8 != 0) {
            std::printf("FAIL column item %d: entry base %d not a multiple of 8\n", it, I.e_base);
            return 1;
        }
        for (int j = 0; j < I.count; ++j) {
            double t = 0.0;
            for (int kc = 0; kc < I.nkc; ++kc)
                for (int c = 0; c < kPfK; ++c) {
                    const uint8_t* p0 = qraw + I.a_off + size_t(kc) * size_t(I.planes) * kPfPlaneBytes + size_t(j) * kPfK + size_t(c);
                    const int64_t code = code_from(p0, kPfPlaneBytes, I.planes);
                    const int64_t e = int64_t(I.e_base) + int64_t(kc) * kPfK + c;
                    if (code && e >= n) {
                        std::printf("FAIL column item %d: code past the matrix\n", it);
                        return 1;
                    }
                    if (e < n) t += double(code) * xc[size_t(e)];
                }
            const PfComp& C = comps[I.comp0 + j];
            for (int d = 0; d < C.ndest; ++d) {
                const int32_t slot = dests[C.dest0 + d] & 0x0FFFFFFF, P = (dests[C.dest0 + d] >> 28) + 1;
                U[size_t(slot)] = C.scale * t;
                ++fed[size_t(slot)];
                slot_planes.resize(std::max(slot_planes.size(), size_t(slot) + 1), 0);
                slot_planes[size_t(slot)] = P;
            }
        }
        // rows past count hold code 0
        for (int kc = 0; kc < I.nkc; ++kc)
            for (int mm = 0; mm < I.planes; ++mm)
                for (int j = I.count; j < kPfM; ++j)
                    for (int c = 0; c < kPfK; ++c)
                        if (qraw[I.a_off + (size_t(kc) * size_t(I.planes) + size_t(mm)) * kPfPlaneBytes + size_t(j) * kPfK + size_t(c)]) {
                            std::printf("FAIL column item %d: padding row %d nonzero\n", it, j);
                            return 1;
                        }
    }

    // row side
    const auto* ri = sec<PfRowItem>(L, L.sec.row_items);
    const auto* rs = sec<int32_t>(L, L.sec.row_sched);
    if (rs[0] != 0 || rs[L.grid] != L.n_row_items) {
        std::printf("FAIL row schedule offsets\n");
        return 1;
    }
    const auto* ch = sec<PfRowChunk>(L, L.sec.chunks);
    const uint8_t* praw = L.arena.data() + L.sec.praw;
    std::vector<double> part(size_t(L.n_parts) * kPfM, 0.0);
    std::vector<int> part_seen(size_t(L.n_parts), 0);
    std::vector<int> chunk_seen(size_t(L.n_chunks), 0);
    double xmax = 0.0;
    for (int64_t e = 0; e < n; ++e) xmax = std::max(xmax, std::fabs(xc[size_t(e)]));
    for (int32_t it = 0; it < L.n_row_items; ++it) {
        const PfRowItem& I = ri[it];
        ++part_seen[size_t(I.part)];
        if (I.u_beta > L.u_beta) {
            std::printf("FAIL row item %d: bound %d above the layout's %d\n", it, I.u_beta, L.u_beta);
            return 1;
        }
        for (int c = 0; c < I.nchunks; ++c) {
            const PfRowChunk& C = ch[I.chunk0 + c];
            ++chunk_seen[size_t(I.chunk0 + c)];
            if (C.kind == 0) {
                const int stored = C.half == 0 ? 128 : 64, off = C.half == 2 ? 64 : 0;
                for (int r = 0; r < stored; ++r)
                    for (int k = 0; k < kPfK; ++k) {
                        const int64_t code = code_from(praw + C.a_off + size_t(r) * kPfK + size_t(k),
                                                       size_t(stored) * kPfK, C.planes);
                        if (!code) continue;
                        if (k >= C.nvalid) {
                            std::printf("FAIL row chunk %d: code in a padding slot\n", I.chunk0 + c);
                            return 1;
                        }
                        if (!fed[size_t(C.b + k)]) {
                            std::printf("FAIL slot %d used but never fed\n", C.b + k);
                            return 1;
                        }
                        if (slot_planes[size_t(C.b + k)] != C.planes) {
                            std::printf("FAIL slot %d: dest planes %d, chunk planes %d\n", C.b + k,
                                        slot_planes[size_t(C.b + k)], C.planes);
                            return 1;
                        }
                        // the item's own bound holds for every slot it reads:
                        // |u| 256^(P-1) < 2^u_beta max|x|
                        if (std::fabs(U[size_t(C.b + k)]) * std::ldexp(1.0, 8 * (C.planes - 1)) >=
                            std::ldexp(xmax, I.u_beta)) {
                            std::printf("FAIL slot %d: |u| above its row item's bound\n", C.b + k);
                            return 1;
                        }
                        part[size_t(I.part) * kPfM + size_t(off + r)] += double(code) * U[size_t(C.b + k)];
                    }
            } else {
                if (C.b % 8 != 0) {
                    std::printf("FAIL dense chunk entry %d not a multiple of 8\n", C.b);
                    return 1;
                }
                const double sc = std::ldexp(1.0, I.dense_exp);
                for (int r = 0; r < kPfM; ++r)
                    for (int k = 0; k < kPfK; ++k) {
                        double v = 0.0;
                        for (int l = 0; l < 3; ++l) {
                            uint16_t h;
                            std::memcpy(&h, praw + C.a_off + size_t(l) * kPfTileBytes + swz(r, k), 2);
                            v += f16_to_double(h);
                        }
                        if (v != 0.0) part[size_t(I.part) * kPfM + size_t(r)] += v * sc * xc[size_t(C.b + k)];
                    }
            }
        }
    }
    for (int32_t c = 0; c < L.n_chunks; ++c)
        if (chunk_seen[size_t(c)] != 1) {
            std::printf("FAIL chunk %d walked %d times\n", c, chunk_seen[size_t(c)]);
            return 1;
        }
    for (int32_t pi = 0; pi < L.n_parts; ++pi)
        if (part_seen[size_t(pi)] != 1) {
            std::printf("FAIL partial %d written %d times\n", pi, part_seen[size_t(pi)]);
            return 1;
        }
    for (int64_t row = 0; row < n; ++row) {
        const int64_t t = row / kPfM;
        double s = 0.0;
        for (int32_t h = L.tile_part0[size_t(t)]; h < L.tile_part0[size_t(t) + 1]; ++h)
            s += part[size_t(h) * kPfM + size_t(row % kPfM)];
        y[size_t(perm[row])] = s;
    }
    std::ofstream fy(argv[3], std::ios::binary);
    fy.write(reinterpret_cast<const char*>(y.data()), std::streamsize(8 * n));
    std::printf("OK items %d/%d chunks %d slots %d parts %d stored %llu/%llu/%llu\n", L.n_col_items, L.n_row_items,
                L.n_chunks, L.n_slots, L.n_parts, (unsigned long long)L.stored_q, (unsigned long long)L.stored_p,
                (unsigned long long)L.stored_dense);
    return 0;
}
