// GB300 (sm_103a) resident quantized H-matrix matvec and its C ABI.
//
// y = A x for a matrix held as dense FP64 diagonal blocks plus low-rank blocks
// whose balanced factors P (rows) and Q (columns) are stored as per-component
// signed integer codes of width w_j in [2, 32], bit-packed LSB-first exactly
// as the reference packs them (src/qhmat/core.cpp:235-267), with one FP64
// scale per factor and component.
//
// FP64 throughput on GB300 is a small fraction of its integer throughput, so
// the per-code arithmetic is exact integer arithmetic and FP64 is used only
// per component, per output row and for the dense diagonal blocks:
//
//   prep_x    x (source order) -> clustered order, fixed point: each chunk of
//             32 clustered entries gets one exponent e and entries
//             X = round(x * 2^(54-e)), |X| <= 2^54.
//   column    t_bj = sum_k cQ_kj X_k, exact in integers (codes times the two
//   side      27-bit limbs of X, int64 accumulation, carry-normalised into a
//             two-word (H, L) integer), then one conversion per component:
//             u_bj = (s^P_bj s^Q_bj) * t_bj * 2^(...)  (FP64).
//             The block's u_bj are then put in fixed point on the block's own
//             exponent (its largest |u_bj|): U_bj, two 27-bit limbs.
//   row side  per tile of <= 64 rows of one elementary row slab: for every
//             block covering the slab, sum_j cP_ij U_bj exactly in integers,
//             shifted onto the tile's exponent with 16 guard bits into a
//             128-bit accumulator; dense diagonal rows in FP64; one conversion
//             per row; one writer per y entry (deterministic, no atomics).
//
// The only rounding steps are the fixed-point conversions of x (2^-55 relative
// to the block's largest |x|) and u (2^-55 relative to the block's largest
// |u|), the product s^P s^Q, the alignment of blocks more than 2^16 below the
// tile's largest, and the final
// FP64 conversions: the result agrees with the reference's FP64 matmul
// (src/qhmat/core.cpp:360-390) to ~1e-15 relative in norm.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/qhmat_gb300.h"
#include "layout.hpp"

namespace qhg {
namespace {

// Fixed point: |X|, |U| <= 2^kFixBits, split into two kLimb-bit limbs
// (low limb unsigned, high limb signed).  A code (|c| < 2^31) times a limb is
// < 2^58, so an int64 accumulator takes kFoldEvery products before it must be
// folded into the two-word (H, L) integer.
constexpr int kFixBits = 54;
constexpr int kLimb = 27;
constexpr long long kLimbMask = (1LL << kLimb) - 1;
constexpr int kFoldEvery = 32;

// ---------------------------------------------------------------- helpers

// Biased IEEE exponent field; 0 for zero/subnormal.  |v| < 2^(e - 1022).
__device__ __forceinline__ int exp_field(double v) {
    return int((__double_as_longlong(v) >> 52) & 0x7FF);
}

// round(v * 2^(kFixBits - (emax - 1022))) as an integer, computed with integer
// operations only (the FP64 pipe is the scarce one).  emax must be >= the
// exponent field of v; subnormals give 0.
__device__ __forceinline__ long long to_fixed(double v, int emax) {
    const long long bits = __double_as_longlong(v);
    const int e = int((bits >> 52) & 0x7FF);
    if (e == 0) return 0;
    const long long mant = (bits & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL;
    // v = mant * 2^(e-1075);  scaled = mant * 2^(e - 1075 + kFixBits - emax + 1022)
    const int rs = emax - e + (1075 - 1022 - kFixBits);  // right shift, >= 53 - kFixBits
    long long q;
    if (rs <= 0) q = mant << (-rs);
    else q = rs >= 62 ? 0 : ((mant + (1LL << (rs - 1))) >> rs);
    return bits < 0 ? -q : q;
}

// Code of entry `row` of a component run starting at word `off`, width w:
// LSB-first bit field at position row*w, sign-extended (the inverse of
// HMatrix::pack, as HMatrix::decode reads it: core.cpp:269-282).
__device__ __forceinline__ int extract_code(const uint32_t* __restrict__ words, uint32_t off,
                                            int row, int w) {
    const uint32_t pos = uint32_t(row) * uint32_t(w);
    const uint32_t wi = off + (pos >> 5);
    const uint32_t lo = __ldg(words + wi);
    const uint32_t hi = __ldg(words + wi + 1);
    const uint32_t raw = __funnelshift_r(lo, hi, pos & 31);
    return int(raw << (32 - w)) >> (32 - w);
}

// (hi * 2^kLimb + lo) added into the two-word integer H * 2^32 + L.
__device__ __forceinline__ void fold(long long hi, long long lo, long long& H, long long& L) {
    H += (hi >> (32 - kLimb)) + (lo >> 32);
    L += ((hi & ((1LL << (32 - kLimb)) - 1)) << kLimb) + (lo & 0xFFFFFFFFLL);
}

__device__ __forceinline__ double two_word_to_double(long long H, long long L) {
    return fma(double(H), 4294967296.0, double(L));
}

struct Arena {
    const int32_t* perm;
    const LowRankDesc* lr;
    const DenseDesc* dd;
    const uint8_t* comp_w;
    const double* comp_s;
    const uint32_t* comp_qoff;
    const uint32_t* comp_poff;
    const uint32_t* qwords;
    const uint32_t* pwords;
    const double* dense;
    const int32_t* a_order;
    const RowTile* tiles;
    const int32_t* items;
};

struct Work {
    long long* X;   // [rhs][n]        fixed-point x, clustered order
    int* xexp;      // [rhs][n_chunks] exponent field of each 32-entry chunk
    double* u;      // [rhs][n_comp]   u_bj = s^P s^Q t_bj (FP64)
    int2* U;        // [rhs][n_comp]   u_bj in fixed point on its block's exponent, two limbs
    int* ub;        // [rhs][n_lr]     exponent field of each block's largest |u_bj|
};

// Guard bits of the row accumulator: a block whose largest |u| is within
// 2^kGuard of the tile's largest is added without rounding.
constexpr int kGuard = 16;

// ---------------------------------------------------------------- kernels

// One warp per (chunk of 32 clustered positions, rhs column).
__global__ void __launch_bounds__(256) prep_x_kernel(Arena A, Work W, const double* __restrict__ x,
                                                     int n, int rhs, int n_chunks, int* status) {
    const int lane = threadIdx.x & 31;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const long long total = (long long)n_chunks * rhs;
    if (gw >= total) return;
    const int p = int(gw / n_chunks), chunk = int(gw % n_chunks);
    const int pos = chunk * kChunk + lane;
    const bool valid = pos < n;
    const double v = valid ? __ldg(x + (long long)__ldg(A.perm + pos) * rhs + p) : 0.0;
    const int e = exp_field(v);
    if (__any_sync(0xFFFFFFFFu, e == 0x7FF) && lane == 0 && status) *status = 1;
    const int emax = __reduce_max_sync(0xFFFFFFFFu, e == 0x7FF ? 0 : e);
    if (valid) W.X[(long long)p * n + pos] = (e == 0x7FF || emax == 0) ? 0 : to_fixed(v, emax);
    if (lane == 0) W.xexp[p * n_chunks + chunk] = emax;
}

// Column side: one warp per low-rank block at a time (persistent warps over
// the blocks, heaviest first).  Lanes own entries k = lane + 32 e; components
// are processed eight at a time and reduced across the warp with a transposed
// multi-reduction (lane l ends up holding component l >> 2).
__global__ void __launch_bounds__(256) column_kernel(Arena A, Work W, int n_a, int n, int rhs,
                                                     int n_chunks, int n_comp, int n_lr) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int wi = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wi < n_a; wi += warps) {
        const LowRankDesc d = A.lr[__ldg(A.a_order + wi)];
        // Block exponent: max chunk exponent over the block's columns.
        const int c_first = d.col0 / kChunk, c_last = (d.col0 + d.n - 1) / kChunk;
        for (int p = 0; p < rhs; ++p) {
            int eb = 0;
            for (int c = c_first + lane; c <= c_last; c += 32) eb = max(eb, __ldg(W.xexp + p * n_chunks + c));
            eb = __reduce_max_sync(0xFFFFFFFFu, eb);
            const long long* Xp = W.X + (long long)p * n;
            const int* Ep = W.xexp + p * n_chunks;
            for (int g = 0; g < d.rank; g += 8) {
                const int gcount = min(8, d.rank - g);
                long long H[8], L[8];
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) H[jj] = L[jj] = 0;
                int wj[8];
                uint32_t oj[8];
#pragma unroll
                for (int jj = 0; jj < 8; ++jj) {
                    const int c = d.comp0 + g + min(jj, gcount - 1);
                    wj[jj] = __ldg(A.comp_w + c);
                    oj[jj] = __ldg(A.comp_qoff + c);
                }
                for (int k0 = 0; k0 < d.n; k0 += 32 * kFoldEvery) {
                    long long ahi[8], alo[8];
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj) ahi[jj] = alo[jj] = 0;
                    const int k1 = min(d.n, k0 + 32 * kFoldEvery);
                    for (int k = k0 + lane; k < k1; k += 32) {
                        const int col = d.col0 + k;
                        long long X = Xp[col];
                        const int sh = eb - Ep[col / kChunk];
                        X = sh >= 63 ? 0 : (sh > 0 ? ((X + (1LL << (sh - 1))) >> sh) : X);
                        const int xl = int(X & kLimbMask);
                        const int xh = int(X >> kLimb);
#pragma unroll
                        for (int jj = 0; jj < 8; ++jj) {
                            if (jj < gcount) {
                                const int code = extract_code(A.qwords, oj[jj], k, wj[jj]);
                                alo[jj] += (long long)code * xl;
                                ahi[jj] += (long long)code * xh;
                            }
                        }
                    }
#pragma unroll
                    for (int jj = 0; jj < 8; ++jj) fold(ahi[jj], alo[jj], H[jj], L[jj]);
                }
                // Transposed reduction: 8 (H, L) pairs over 32 lanes.
                {
                    const bool b4 = lane & 16;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const long long sh_ = b4 ? H[i] : H[i + 4], sl = b4 ? L[i] : L[i + 4];
                        const long long rh = __shfl_xor_sync(0xFFFFFFFFu, sh_, 16);
                        const long long rl = __shfl_xor_sync(0xFFFFFFFFu, sl, 16);
                        H[i] = (b4 ? H[i + 4] : H[i]) + rh;
                        L[i] = (b4 ? L[i + 4] : L[i]) + rl;
                    }
                    const bool b3 = lane & 8;
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        const long long sh_ = b3 ? H[i] : H[i + 2], sl = b3 ? L[i] : L[i + 2];
                        const long long rh = __shfl_xor_sync(0xFFFFFFFFu, sh_, 8);
                        const long long rl = __shfl_xor_sync(0xFFFFFFFFu, sl, 8);
                        H[i] = (b3 ? H[i + 2] : H[i]) + rh;
                        L[i] = (b3 ? L[i + 2] : L[i]) + rl;
                    }
                    const bool b2 = lane & 4;
                    {
                        const long long sh_ = b2 ? H[0] : H[1], sl = b2 ? L[0] : L[1];
                        const long long rh = __shfl_xor_sync(0xFFFFFFFFu, sh_, 4);
                        const long long rl = __shfl_xor_sync(0xFFFFFFFFu, sl, 4);
                        H[0] = (b2 ? H[1] : H[0]) + rh;
                        L[0] = (b2 ? L[1] : L[0]) + rl;
                    }
                    H[0] += __shfl_xor_sync(0xFFFFFFFFu, H[0], 2);
                    L[0] += __shfl_xor_sync(0xFFFFFFFFu, L[0], 2);
                    H[0] += __shfl_xor_sync(0xFFFFFFFFu, H[0], 1);
                    L[0] += __shfl_xor_sync(0xFFFFFFFFu, L[0], 1);
                }
                const int jj = lane >> 2;  // component held by this lane
                if ((lane & 3) == 0 && jj < gcount) {
                    const int c = d.comp0 + g + jj;
                    // x ~= X * 2^(eb - 1022 - kFixBits) after alignment.
                    const double t = scalbn(two_word_to_double(H[0], L[0]), eb - 1022 - kFixBits);
                    W.u[(long long)p * n_comp + c] = t * __ldg(A.comp_s + c);
                }
            }
            __syncwarp();
            // The block's u on one fixed-point exponent (its largest |u_bj|).
            double* up = W.u + (long long)p * n_comp + d.comp0;
            int e = 0;
            for (int j = lane; j < d.rank; j += 32) e = max(e, exp_field(up[j]));
            e = __reduce_max_sync(0xFFFFFFFFu, e);
            int2* Up = W.U + (long long)p * n_comp + d.comp0;
            for (int j = lane; j < d.rank; j += 32) {
                const long long v = e ? to_fixed(up[j], e) : 0;
                Up[j] = make_int2(int(v & kLimbMask), int(v >> kLimb));
            }
            if (lane == 0) W.ub[(long long)p * n_lr + __ldg(A.a_order + wi)] = e;
        }
    }
}

// Row side: one CTA of kTileRows threads per row tile; thread t owns clustered
// row tile.row0 + t.  For each low-rank block covering the tile the row's
// sum_j cP_ij U_bj is formed exactly (U_bj on the block's own exponent), then
// shifted onto the tile's exponent (largest block exponent, kGuard guard
// bits) and added into a 128-bit accumulator.  Dense diagonal rows are FP64.
__global__ void __launch_bounds__(kTileRows) row_kernel(Arena A, Work W, const double* __restrict__ x,
                                                        double* __restrict__ y, int n, int rhs,
                                                        int n_comp, int n_lr) {
    __shared__ int s_emax[kTileRows / 32];
    const RowTile T = A.tiles[blockIdx.x];
    const int t = threadIdx.x;
    const bool active = t < T.rows;
    const int row = T.row0 + t;
    for (int p = 0; p < rhs; ++p) {
        const int* ub = W.ub + (long long)p * n_lr;
        const int2* Up = W.U + (long long)p * n_comp;
        // 1. tile exponent: the largest block exponent among the tile's items.
        int emax = 0;
        for (int it = T.item0 + t; it < T.item1; it += blockDim.x) {
            const int item = __ldg(A.items + it);
            if (item >= 0 && A.lr[item].rank > 0) emax = max(emax, ub[item]);
        }
        emax = __reduce_max_sync(0xFFFFFFFFu, emax);
        if ((t & 31) == 0) s_emax[t >> 5] = emax;
        __syncthreads();
        emax = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) emax = max(emax, s_emax[i]);
        // 2. accumulate.
        __int128 acc = 0;
        double diag = 0.0;
        for (int it = T.item0; it < T.item1; ++it) {
            const int item = __ldg(A.items + it);
            if (!active) continue;
            if (item >= 0) {
                const LowRankDesc d = A.lr[item];
                if (d.rank == 0) continue;
                const int rloc = row - d.row0;
                __int128 vb = 0;
                long long ahi = 0, alo = 0;
                int cnt = 0;
                for (int j = 0; j < d.rank; ++j) {
                    const int c = d.comp0 + j;
                    const int code = extract_code(A.pwords, __ldg(A.comp_poff + c), rloc, __ldg(A.comp_w + c));
                    const int2 U = Up[c];
                    alo += (long long)code * U.x;
                    ahi += (long long)code * U.y;
                    if (++cnt == kFoldEvery) {
                        vb += ((__int128)ahi << kLimb) + alo;
                        ahi = alo = 0;
                        cnt = 0;
                    }
                }
                vb += ((__int128)ahi << kLimb) + alo;
                const int sh = (emax - ub[item]) - kGuard;
                if (sh <= 0) acc += vb << (-sh);
                else if (sh < 127) acc += (vb + ((__int128)1 << (sh - 1))) >> sh;
            } else {
                const DenseDesc d = A.dd[-1 - item];
                const double* Drow = A.dense + d.off + (long long)(row - d.row0) * d.n;
                for (int k = 0; k < d.n; ++k)
                    diag = fma(__ldg(Drow + k), __ldg(x + (long long)__ldg(A.perm + d.col0 + k) * rhs + p), diag);
            }
        }
        if (active) {
            double lr = 0.0;
            if (emax) {
                const long long hi = (long long)(acc >> 64);
                const unsigned long long lo = (unsigned long long)acc;
                lr = scalbn(fma(double(hi), 18446744073709551616.0, double(lo)), emax - 1022 - kFixBits - kGuard);
            }
            y[(long long)__ldg(A.perm + row) * rhs + p] = diag + lr;
        }
        __syncthreads();
    }
}

// Validation: decode every code of one side, one warp per component.
__global__ void decode_kernel(Arena A, int side, int n_lr, const long long* __restrict__ out_off,
                              int* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < n_lr; b += warps) {
        const LowRankDesc d = A.lr[b];
        const int rows = side == 0 ? d.m : d.n;
        const uint32_t* words = side == 0 ? A.pwords : A.qwords;
        const uint32_t* offs = side == 0 ? A.comp_poff : A.comp_qoff;
        long long o = out_off[b];
        for (int j = 0; j < d.rank; ++j) {
            const int c = d.comp0 + j;
            for (int i = lane; i < rows; i += 32) out[o + i] = extract_code(words, offs[c], i, A.comp_w[c]);
            o += rows;
        }
    }
}

// ---------------------------------------------------------------- host side

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(QH_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

}  // namespace
}  // namespace qhg

using namespace qhg;

struct qh_matrix {
    Layout L;
    int device = 0;
    int sms = 1;
    void* arena = nullptr;  // device copy of L.arena
    Arena A{};
    // lazily allocated scratch for calls without a workspace, and host staging
    std::mutex mu;
    void* own_ws = nullptr;
    size_t own_ws_bytes = 0;
    double* pinned = nullptr;
    size_t pinned_bytes = 0;
    int* d_status = nullptr;
    int* h_status = nullptr;
    cudaStream_t stream = nullptr;
    ~qh_matrix() {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        if (arena) cudaFree(arena);
        if (own_ws) cudaFree(own_ws);
        if (d_status) cudaFree(d_status);
        if (pinned) cudaFreeHost(pinned);
        if (h_status) cudaFreeHost(h_status);
        if (stream) cudaStreamDestroy(stream);
        cudaSetDevice(prev);
    }
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int check_device(int device) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (!count) return fail(QH_ERUNTIME, "no CUDA device is available");
    if (device < 0 || device >= count) return fail(QH_EINVAL, "invalid CUDA device ordinal");
    return QH_OK;
}

int upload(Layout&& L, int device, qh_matrix** out) {
    int rc = check_device(device);
    if (rc) return rc;
    DeviceGuard g(device);
    qh_matrix* m = new (std::nothrow) qh_matrix();
    if (!m) return fail(QH_ERUNTIME, "out of host memory");
    m->L = std::move(L);
    m->device = device;
    cudaError_t e = cudaMalloc(&m->arena, m->L.sec.total);
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "cudaMalloc");
    }
    e = cudaMemcpy(m->arena, m->L.arena.data(), m->L.sec.total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "cudaMemcpy host-to-device");
    }
    cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
    // The host image is no longer needed once uploaded.
    std::vector<uint8_t>().swap(m->L.arena);
    const Sections& S = m->L.sec;
    auto* base = static_cast<const uint8_t*>(m->arena);
    m->A.perm = reinterpret_cast<const int32_t*>(base + S.perm);
    m->A.lr = reinterpret_cast<const LowRankDesc*>(base + S.lr);
    m->A.dd = reinterpret_cast<const DenseDesc*>(base + S.dd);
    m->A.comp_w = base + S.comp_w;
    m->A.comp_s = reinterpret_cast<const double*>(base + S.comp_s);
    m->A.comp_qoff = reinterpret_cast<const uint32_t*>(base + S.comp_qoff);
    m->A.comp_poff = reinterpret_cast<const uint32_t*>(base + S.comp_poff);
    m->A.qwords = reinterpret_cast<const uint32_t*>(base + S.qwords);
    m->A.pwords = reinterpret_cast<const uint32_t*>(base + S.pwords);
    m->A.dense = reinterpret_cast<const double*>(base + S.dense);
    m->A.a_order = reinterpret_cast<const int32_t*>(base + S.a_order);
    m->A.tiles = reinterpret_cast<const RowTile*>(base + S.tiles);
    m->A.items = reinterpret_cast<const int32_t*>(base + S.items);
    *out = m;
    return QH_OK;
}

template <class F>
int guarded(F&& f) {
    try {
        return f();
    } catch (const std::invalid_argument& e) {
        return fail(QH_EINVAL, e.what());
    } catch (const std::overflow_error& e) {
        return fail(QH_EOVERFLOW, e.what());
    } catch (const std::bad_alloc&) {
        return fail(QH_ERUNTIME, "out of host memory");
    } catch (const std::exception& e) {
        return fail(QH_ERUNTIME, e.what());
    }
}

struct WsPlan {
    size_t X, xexp, u, U, ub, total;
};

WsPlan ws_plan(const Layout& L, size_t rhs) {
    WsPlan w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += align256(std::max<size_t>(bytes, 1));
        return o;
    };
    w.X = take(8 * L.order * rhs);
    w.xexp = take(4 * size_t(L.n_chunks) * rhs);
    w.u = take(8 * size_t(L.n_comp) * rhs);
    w.U = take(8 * size_t(L.n_comp) * rhs);
    w.ub = take(4 * size_t(L.n_lr) * rhs);
    w.total = off;
    return w;
}

size_t ws_bytes(const Layout& L, size_t rhs) { return ws_plan(L, rhs).total; }

int launch(const qh_matrix* m, const double* x, double* y, size_t rhs, void* ws, cudaStream_t s,
           int* status, void* const* ev = nullptr) {
    const Layout& L = m->L;
    const int n = int(L.order);
    auto* w = static_cast<uint8_t*>(ws);
    const WsPlan P = ws_plan(L, rhs);
    Work W;
    W.X = reinterpret_cast<long long*>(w + P.X);
    W.xexp = reinterpret_cast<int*>(w + P.xexp);
    W.u = reinterpret_cast<double*>(w + P.u);
    W.U = reinterpret_cast<int2*>(w + P.U);
    W.ub = reinterpret_cast<int*>(w + P.ub);
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[i]), s);
    };
    const long long prep_warps = (long long)L.n_chunks * (long long)rhs;
    mark(0);
    prep_x_kernel<<<unsigned((prep_warps + 7) / 8), 256, 0, s>>>(m->A, W, x, n, int(rhs), L.n_chunks, status);
    mark(1);
    if (L.n_a > 0) {
        const int grid = std::max(1, std::min((L.n_a + 7) / 8, m->sms * 8));
        column_kernel<<<grid, 256, 0, s>>>(m->A, W, L.n_a, n, int(rhs), L.n_chunks, L.n_comp, L.n_lr);
    }
    mark(2);
    row_kernel<<<L.n_tiles, kTileRows, 0, s>>>(m->A, W, x, y, n, int(rhs), L.n_comp, L.n_lr);
    mark(3);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "CUDA kernel launch");
    return QH_OK;
}

int check_rhs(const qh_matrix* m, size_t rhs) {
    if (rhs == 0 || rhs > SIZE_MAX / m->L.order / 8) return fail(QH_EINVAL, "right-hand-side shape mismatch");
    if (rhs > size_t(INT32_MAX) || m->L.order * rhs > (size_t(1) << 40))
        return fail(QH_EOVERFLOW, "CUDA launch grid too large");
    return QH_OK;
}

}  // namespace

extern "C" {

const char* qh_last_error(void) { return g_last_error.c_str(); }

int qh_cuda_built(void) { return 1; }

int qh_matrix_from_qhmat(const void* bytes, size_t len, int device, qh_matrix** out) {
    if (!out) return fail(QH_EINVAL, "output handle pointer is null");
    *out = nullptr;
    if (!bytes && len) return fail(QH_EINVAL, "image pointer is null");
    return guarded([&] {
        HostMatrix hm = parse_qhmat(static_cast<const uint8_t*>(bytes), len);
        Layout L = build_layout(hm);
        return upload(std::move(L), device, out);
    });
}

int qh_matrix_from_arrays(size_t order, const size_t* permutation, size_t block_count,
                          const qh_block_desc* blocks, const double* dense,
                          const uint32_t* left_words, const uint32_t* right_words,
                          const size_t* left_offsets, const size_t* right_offsets,
                          const double* left_scales, const double* right_scales, const int* widths,
                          int device, qh_matrix** out) {
    if (!out) return fail(QH_EINVAL, "output handle pointer is null");
    *out = nullptr;
    if (!order || !permutation || !block_count || !blocks)
        return fail(QH_EINVAL, "invalid matrix order/permutation");
    return guarded([&] {
        HostMatrix hm;
        hm.order = order;
        hm.permutation.assign(permutation, permutation + order);
        size_t n_comp = 0, n_dense = 0, lw_end = 0, rw_end = 0;
        for (size_t k = 0; k < block_count; ++k) {
            const auto& d = blocks[k];
            HostMatrix::Block b;
            b.row0 = d.row0;
            b.row1 = d.row1;
            b.col0 = d.col0;
            b.col1 = d.col1;
            b.admissible = false;
            b.dense = d.is_dense != 0;
            if (d.row1 < d.row0 || d.col1 < d.col0) throw std::invalid_argument("invalid block rectangle");
            if (b.dense) {
                b.dense_off = d.dense_offset;
                n_dense = std::max(n_dense, d.dense_offset + (d.row1 - d.row0) * (d.col1 - d.col0));
            } else {
                b.rank = d.rank;
                b.comp0 = d.factor_offset;
                n_comp = std::max(n_comp, d.factor_offset + d.rank);
                for (size_t j = 0; j < d.rank; ++j) {
                    const size_t c = d.factor_offset + j;
                    const int w = widths[c];
                    if (w < 2 || w > 32) throw std::invalid_argument("bit width must be in [2, 32]");
                    lw_end = std::max(lw_end, left_offsets[c] + ((d.row1 - d.row0) * size_t(w) + 31) / 32);
                    rw_end = std::max(rw_end, right_offsets[c] + ((d.col1 - d.col0) * size_t(w) + 31) / 32);
                }
            }
            hm.blocks.push_back(b);
        }
        if (n_dense && !dense) throw std::invalid_argument("dense values pointer is null");
        hm.dense.assign(dense, dense + n_dense);
        if (n_comp && (!widths || !left_scales || !right_scales || !left_offsets || !right_offsets ||
                       !left_words || !right_words))
            throw std::invalid_argument("factor arrays are null");
        hm.width.resize(n_comp);
        for (size_t c = 0; c < n_comp; ++c) hm.width[c] = uint8_t(widths[c]);
        hm.left_scale.assign(left_scales, left_scales + n_comp);
        hm.right_scale.assign(right_scales, right_scales + n_comp);
        hm.left_off.assign(left_offsets, left_offsets + n_comp);
        hm.right_off.assign(right_offsets, right_offsets + n_comp);
        hm.left_words.assign(left_words, left_words + lw_end);
        hm.right_words.assign(right_words, right_words + rw_end);
        validate(hm);
        Layout L = build_layout(hm);
        return upload(std::move(L), device, out);
    });
}

void qh_matrix_destroy(qh_matrix* m) { delete m; }

int qh_matrix_stats(const qh_matrix* m, qh_stats* out) {
    if (!m || !out) return fail(QH_EINVAL, "null argument");
    const Layout& L = m->L;
    out->order = L.order;
    out->block_count = uint64_t(L.n_lr) + uint64_t(L.n_dense);
    out->dense_blocks = uint64_t(L.n_dense);
    out->lowrank_blocks = uint64_t(L.n_lr);
    out->components = uint64_t(L.n_comp);
    out->code_bytes = L.code_bytes;
    out->scale_bytes = L.scale_bytes;
    out->dense_bytes = L.dense_bytes;
    out->model_bytes = L.code_bytes + L.scale_bytes + L.dense_bytes + 16 * L.order;
    out->device_bytes = L.sec.total;
    out->row_tiles = uint64_t(L.n_tiles);
    out->flops_per_rhs = L.flops;
    return QH_OK;
}

double qh_matrix_reconstruction_bound(const qh_matrix* m) { return m ? m->L.bound : 0.0; }

size_t qh_workspace_bytes(const qh_matrix* m, size_t rhs) { return m ? ws_bytes(m->L, rhs) : 0; }

int qh_matmul_device(const qh_matrix* m, const double* x, double* y, size_t rhs, void* workspace,
                     size_t workspace_bytes, void* stream, int* status) {
    return qh_matmul_device_profiled(m, x, y, rhs, workspace, workspace_bytes, stream, status, nullptr);
}

int qh_matmul_device_profiled(const qh_matrix* m, const double* x, double* y, size_t rhs, void* workspace,
                              size_t workspace_bytes, void* stream, int* status, void* const* events4) {
    if (!m) return fail(QH_EINVAL, "null matrix handle");
    int rc = check_rhs(m, rhs);
    if (rc) return rc;
    if (!x || !y) return fail(QH_EINVAL, "null right-hand side or result pointer");
    DeviceGuard g(m->device);
    const size_t need = ws_bytes(m->L, rhs);
    if (workspace) {
        if (workspace_bytes < need) return fail(QH_EINVAL, "workspace too small");
        if (reinterpret_cast<uintptr_t>(workspace) & 255) return fail(QH_EINVAL, "workspace must be 256-byte aligned");
        return launch(m, x, y, rhs, workspace, static_cast<cudaStream_t>(stream), status, events4);
    }
    auto* mm = const_cast<qh_matrix*>(m);
    std::lock_guard<std::mutex> lock(mm->mu);
    if (mm->own_ws_bytes < need) {
        if (mm->own_ws) cudaFree(mm->own_ws);
        mm->own_ws = nullptr;
        mm->own_ws_bytes = 0;
        cudaError_t e = cudaMalloc(&mm->own_ws, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        mm->own_ws_bytes = need;
    }
    return launch(m, x, y, rhs, mm->own_ws, static_cast<cudaStream_t>(stream), status, events4);
}

int qh_matmul_host(const qh_matrix* m, const double* x, double* y, size_t rhs) {
    if (!m) return fail(QH_EINVAL, "null matrix handle");
    int rc = check_rhs(m, rhs);
    if (rc) return rc;
    rc = check_device(m->device);
    if (rc) return rc;
    if (!x || !y) return fail(QH_EINVAL, "null right-hand side or result pointer");
    auto* mm = const_cast<qh_matrix*>(m);
    DeviceGuard g(m->device);
    std::lock_guard<std::mutex> lock(mm->mu);
    cudaError_t e;
    if (!mm->stream) {
        e = cudaStreamCreateWithFlags(&mm->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    }
    if (!mm->d_status) {
        e = cudaMalloc(&mm->d_status, sizeof(int));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        e = cudaMallocHost(&mm->h_status, sizeof(int));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
    }
    const size_t vec = m->L.order * rhs * sizeof(double);
    const size_t need_ws = ws_bytes(m->L, rhs);
    // one device buffer: workspace | x | y
    const size_t need = align256(need_ws) + 2 * align256(vec);
    if (mm->own_ws_bytes < need) {
        if (mm->own_ws) cudaFree(mm->own_ws);
        mm->own_ws = nullptr;
        mm->own_ws_bytes = 0;
        e = cudaMalloc(&mm->own_ws, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        mm->own_ws_bytes = need;
    }
    if (mm->pinned_bytes < vec) {
        if (mm->pinned) cudaFreeHost(mm->pinned);
        mm->pinned = nullptr;
        mm->pinned_bytes = 0;
        e = cudaMallocHost(&mm->pinned, vec);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost");
        mm->pinned_bytes = vec;
    }
    auto* base = static_cast<uint8_t*>(mm->own_ws);
    double* dx = reinterpret_cast<double*>(base + align256(need_ws));
    double* dy = reinterpret_cast<double*>(base + align256(need_ws) + align256(vec));
    std::memcpy(mm->pinned, x, vec);
    if ((e = cudaMemsetAsync(mm->d_status, 0, sizeof(int), mm->stream)) != cudaSuccess)
        return cuda_fail(e, "cudaMemsetAsync");
    if ((e = cudaMemcpyAsync(dx, mm->pinned, vec, cudaMemcpyHostToDevice, mm->stream)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy host-to-device");
    rc = launch(m, dx, dy, rhs, base, mm->stream, mm->d_status);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(mm->pinned, dy, vec, cudaMemcpyDeviceToHost, mm->stream)) != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy device-to-host");
    if ((e = cudaMemcpyAsync(mm->h_status, mm->d_status, sizeof(int), cudaMemcpyDeviceToHost, mm->stream)) !=
        cudaSuccess)
        return cuda_fail(e, "cudaMemcpy device-to-host");
    if ((e = cudaStreamSynchronize(mm->stream)) != cudaSuccess) return cuda_fail(e, "CUDA kernel execution");
    if (*mm->h_status) return fail(QH_EINVAL, "nonfinite right-hand side");
    std::memcpy(y, mm->pinned, vec);
    return QH_OK;
}

int qh_debug_decode(const qh_matrix* m, int side, int32_t* out, size_t out_count, size_t* needed) {
    if (!m) return fail(QH_EINVAL, "null matrix handle");
    if (side != 0 && side != 1) return fail(QH_EINVAL, "side must be 0 (left) or 1 (right)");
    return guarded([&] {
        // Block offsets into the output, from the host copy of the descriptors.
        DeviceGuard g(m->device);
        std::vector<LowRankDesc> lr(size_t(m->L.n_lr));
        cudaError_t e;
        if (!lr.empty()) {
            e = cudaMemcpy(lr.data(), m->A.lr, sizeof(LowRankDesc) * lr.size(), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy device-to-host");
        }
        std::vector<long long> off(lr.size() + 1, 0);
        for (size_t b = 0; b < lr.size(); ++b)
            off[b + 1] = off[b] + (long long)lr[b].rank * (side == 0 ? lr[b].m : lr[b].n);
        const size_t total = size_t(off.back());
        if (needed) *needed = total;
        if (!out) return QH_OK;
        if (out_count != total) return fail(QH_EINVAL, "output size does not match the code count");
        if (!total) return QH_OK;
        long long* d_off = nullptr;
        int* d_out = nullptr;
        if ((e = cudaMalloc(&d_off, sizeof(long long) * off.size())) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        if ((e = cudaMalloc(&d_out, sizeof(int) * total)) != cudaSuccess) {
            cudaFree(d_off);
            return cuda_fail(e, "cudaMalloc");
        }
        int rc = QH_OK;
        e = cudaMemcpy(d_off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            decode_kernel<<<std::max(1, std::min((m->L.n_lr + 7) / 8, 4096)), 256>>>(m->A, side, m->L.n_lr, d_off, d_out);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(int) * total, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "debug decode");
        cudaFree(d_off);
        cudaFree(d_out);
        return rc;
    });
}

}  // extern "C"
