// GB300 (sm_103a) resident quantized H-matrix matvec and its C ABI.
//
// y = A x for a matrix held as dense FP64 diagonal blocks plus low-rank blocks
// whose balanced factors P (rows) and Q (columns) are stored as per-component
// signed integer codes of width w_j in [2, 32], bit-packed LSB-first exactly
// as the reference packs them (src/qhmat/core.cpp:235-267), with one FP64
// scale per factor and component.  The words are permuted for coalesced
// access (layout.hpp); each code keeps its reference bits.
//
// FP64 throughput on GB300 is a small fraction of its integer throughput, so
// the per-code arithmetic is exact integer arithmetic and FP64 is used only
// per component, per output row and for the dense diagonal blocks:
//
//   prep_x    x (source order) -> clustered order, fixed point: each chunk of
//             32 clustered entries gets one exponent e and entries
//             X = round(x * 2^(54-e)), |X| <= 2^54 (plus an FP64 clustered
//             copy for the dense diagonal blocks).
//   column    one warp per task of <= 32 components sharing a column range
//   side      and a width, one component per lane: t = sum_k cQ_k X_k exactly
//             (codes times the two 27-bit limbs of X, int64 accumulation
//             folded into a two-word integer every 32 entries), then
//             u = (s^P s^Q) * t in FP64, one conversion per component.
//   row side  one CTA per tile of <= 64 rows of one elementary row slab, its
//             eight warps splitting the blocks covering the tile; two rows per
//             lane.  A block's u are put in fixed point on the block's own
//             exponent (U, two 27-bit limbs), sum_j cP_ij U_j is exact, and
//             the block sum is shifted onto the tile's exponent (16 guard
//             bits) into a 128-bit accumulator; dense diagonal rows in FP64;
//             warps combine in shared memory in a fixed order; one writer per
//             y entry (deterministic, no atomics).
//
// The only rounding steps are the fixed-point conversions of x (2^-55 relative
// to the block's largest |x|) and u (2^-55 relative to the block's largest
// |u|), the product s^P s^Q, the alignment of blocks more than 2^16 below the
// tile's largest, and the final FP64 conversions: the result agrees with the
// reference's FP64 matmul (src/qhmat/core.cpp:360-390) to ~1e-15 in norm.
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

// Fixed point: |X|, |U| <= 2^kFixBits, split into two kLimb-bit limbs (low
// limb unsigned, high limb signed).  A code (|c| < 2^31) times a limb is
// < 2^58, so an int64 accumulator takes kFoldEvery products before it is
// folded into a wider integer.
constexpr int kFixBits = 54;
constexpr int kLimb = 27;
constexpr long long kLimbMask = (1LL << kLimb) - 1;
// (kFoldEvery = kColChunk: one column chunk, or 32 row-side components.)
// Guard bits of the row accumulator: a block whose largest |u| is within
// 2^kGuard of the tile's largest is added without rounding.
constexpr int kGuard = 16;


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
    const int rs = emax - e + (1075 - 1022 - kFixBits);  // right shift, >= 53 - kFixBits
    long long q;
    if (rs <= 0) q = mant << (-rs);
    else q = rs >= 62 ? 0 : ((mant + (1LL << (rs - 1))) >> rs);
    return bits < 0 ? -q : q;
}

// Sign-extend the low W bits of r.
template <int W>
__device__ __forceinline__ int sext(uint32_t r) {
    return int(r << (32 - W)) >> (32 - W);
}

// Code e of a bit string held in registers w[0..]: bits [e*W, e*W + W),
// LSB-first -- the field HMatrix::decode reads (core.cpp:269-282).  Called
// from fully unrolled loops, so the word index and shift are constants.
template <int W>
__device__ __forceinline__ int code_at(const uint32_t* w, int e) {
    const int pos = e * W, wi = pos >> 5, off = pos & 31;
    if (off + W <= 32) return sext<W>(w[wi] >> off);
    return sext<W>(__funnelshift_r(w[wi], w[wi + 1], off));
}

// (hi * 2^kLimb + lo) as a 128-bit integer.
__device__ __forceinline__ __int128 widen(long long hi, long long lo) {
    return ((__int128)hi << kLimb) + lo;
}


struct Arena {
    const int32_t* perm;
    const LowRankDesc* lr;
    const DenseDesc* dd;
    const uint8_t* comp_w;
    const double* comp_s;
    const ColTask* tasks;
    const int32_t* task_comp;
    const uint32_t* qwords;
    const uint32_t* pwords;
    const double* dense;
    const RowTile* tiles;
    const RowItem* items;
};

struct Work {
    double* xc;        // [rhs][n]  x in clustered order (FP64)
    int2* xl;          // [rhs][n]  x in fixed point on its column's exponent, two limbs
    int* xe;           // [rhs]     largest exponent field of x (zeroed before prep_x)
    int* split_cnt;    // [n_split][rhs] finished parts of each split column task (zeroed)
    long long* part;   // [n_split][max_parts][rhs][32][2] partial sums of split tasks
    double* u;         // [rhs][n_comp] u_bj = s^P s^Q t_bj (FP64)
};

// -------------------------------------------------- bulk copies (TMA)

__device__ __forceinline__ unsigned smem_u32(const void* p) { return unsigned(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// Arrive once and expect `bytes` more bytes of transactions on this phase.
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up (returns false) after kWaitLimit polls instead of
// hanging; callers record the failure in the status word and stop.
constexpr int kWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    for (int i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Order this thread's (and, after a warp barrier, its warp's) earlier generic
// accesses to shared memory before later asynchronous-proxy writes to it.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// One-dimensional bulk copy global -> shared (16-byte aligned, bytes % 16 == 0),
// completing on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Slot of a warp's prefetch pipeline: up to 4 KB of code words plus up to 33
// doubles (x entries or u values, copied from an 8-byte-aligned start rounded
// down to 16 bytes).
constexpr int kSlotBytes = kStageWordBytes + 272;
constexpr int kStages = 3;
constexpr int kWarps = 8;
constexpr int kPipeSmem = kWarps * kStages * kSlotBytes;

// Status bits written by the kernels (status word of the apply).
constexpr int kStatusNonfinite = 1;
constexpr int kStatusTimeout = 2;

__device__ __forceinline__ void flag_timeout(int* status) {
    if (status) atomicOr(status, kStatusTimeout);
}

// round(v * 2^k) for a 128-bit integer v, as a double, with integer
// operations only (round to nearest even; results outside the normal range
// take the slow path).
__device__ __forceinline__ double i128_ldexp(__int128 v, int k) {
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    const unsigned __int128 a = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    const unsigned long long hi = (unsigned long long)(a >> 64), lo = (unsigned long long)a;
    const int nbits = hi ? 128 - __clzll(hi) : 64 - __clzll(lo);
    unsigned long long mant;
    int e;
    if (nbits <= 53) {
        mant = lo << (53 - nbits);
        e = nbits - 53;
    } else {
        const int sh = nbits - 53;
        const unsigned __int128 q = a >> sh;
        const unsigned __int128 rem = a - (q << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        mant = (unsigned long long)q;
        if (rem > half || (rem == half && (mant & 1))) ++mant;
        e = sh;
        if (mant >> 53) {
            mant >>= 1;
            ++e;
        }
    }
    const int E = e + k + 52 + 1023;
    if (E <= 0 || E >= 2047) return scalbn(neg ? -double(mant) : double(mant), e + k);
    const unsigned long long bits =
        ((unsigned long long)neg << 63) | ((unsigned long long)E << 52) | (mant & 0xFFFFFFFFFFFFFULL);
    return __longlong_as_double((long long)bits);
}

// ------------------------------------------------------------- decoders

// Column side: the 32 codes of lane `lane`'s chunk `ch` of a task (layout.hpp:
// word v of the chunk at q[(ch*W + v)*count + lane]).
template <int W>
__device__ __forceinline__ void col_chunk_words(const uint32_t* __restrict__ q, int ch, int count, int lane,
                                                uint32_t (&w)[W]) {
    const uint32_t* base = q + (size_t)ch * W * count + lane;
#pragma unroll
    for (int v = 0; v < W; ++v) w[v] = __ldg(base + (size_t)v * count);
}

template <int W>
__device__ __forceinline__ void col_chunk_codes(const uint32_t (&w)[W], int (&c)[32]) {
#pragma unroll
    for (int e = 0; e < 32; ++e) c[e] = code_at<W>(w, e);
}

// Row side: codes of rows 2*lane and 2*lane+1 of a piece (the bit string of
// the tile's rows of one component, from a fresh word), width W at run time.
// No branches: three words are read and the shift amounts computed, because a
// data-dependent branch per component stalls the warp far longer than the
// extra arithmetic.
__device__ __forceinline__ void row_pair_codes_rt(const uint32_t* piece, int lane, int W, int& c0, int& c1) {
    const uint32_t pos = uint32_t(lane) * uint32_t(2 * W);
    const uint32_t wi = pos >> 5, off = pos & 31;
    const uint32_t a = piece[wi], b = piece[wi + 1], d = piece[wi + 2];
    const uint32_t sh = 32u - uint32_t(W);
    c0 = int(__funnelshift_r(a, b, off) << sh) >> sh;
    const uint32_t p1 = off + uint32_t(W);
    const uint32_t lo = p1 < 32 ? a : b, hi = p1 < 32 ? b : d;
    c1 = int(__funnelshift_r(lo, hi, p1 & 31) << sh) >> sh;
}

// Dispatch a width to a template instance.
#define QH_WIDTH_CASES(X) \
    X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17) \
    X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31) X(32)

// ---------------------------------------------------------------- kernels

// One warp per (chunk of 32 clustered positions, rhs column): clustered FP64
// copy of x, largest exponent field per column (atomicMax), nonfinite flag.
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
    if (__any_sync(0xFFFFFFFFu, e == 0x7FF) && lane == 0 && status) atomicOr(status, kStatusNonfinite);
    const int emax = __reduce_max_sync(0xFFFFFFFFu, e == 0x7FF ? 0 : e);
    if (valid) W.xc[(long long)p * n + pos] = e == 0x7FF ? 0.0 : v;
    if (lane == 0 && emax) atomicMax(W.xe + p, emax);
}

// x in fixed point on its column's exponent (one thread per entry), after
// prep_x_kernel has found the exponent.
__global__ void __launch_bounds__(256) x_limbs_kernel(Work W, int n, int rhs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)n * rhs) return;
    const int p = int(i / n);
    const int xe = W.xe[p];
    const long long X = xe ? to_fixed(W.xc[i], xe) : 0;
    W.xl[i] = make_int2(int(X & kLimbMask), int(X >> kLimb));
}

// sum_{e<NE} code_e * X_e for NE codes held in registers w[], decoded as
// consumed.
template <int W, int NE>
__device__ __forceinline__ void codes_mac(const uint32_t* w, const int2* sX, long long& alo, long long& ahi) {
    // four independent accumulator pairs keep the multiply-add chains short
    long long l[4] = {0, 0, 0, 0}, h[4] = {0, 0, 0, 0};
#pragma unroll
    for (int e = 0; e < NE; ++e) {
        const int2 xx = sX[e];
        const int c = code_at<W>(w, e);
        l[e & 3] += (long long)c * xx.x;
        h[e & 3] += (long long)c * xx.y;
    }
    alo += (l[0] + l[1]) + (l[2] + l[3]);
    ahi += (h[0] + h[1]) + (h[2] + h[3]);
}

// One 32-entry chunk of a column task from a stage: lane l's words are
// st.words[v * count + l].  Widths above 16 in two halves of 16 codes.
template <int W>
__device__ __forceinline__ void column_chunk(const uint32_t* sw, int count, int lane, const int2* sX,
                                             long long& alo, long long& ahi) {
    const uint32_t* base = sw + lane;
    if constexpr (W <= 16 || (W & 1)) {
        uint32_t w[W];
#pragma unroll
        for (int v = 0; v < W; ++v) w[v] = base[v * count];
        codes_mac<W, 32>(w, sX, alo, ahi);
    } else {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            uint32_t w[W / 2];
#pragma unroll
            for (int v = 0; v < W / 2; ++v) w[v] = base[(h * (W / 2) + v) * count];
            codes_mac<W, 16>(w, sX + 16 * h, alo, ahi);
        }
    }
}

__device__ __noinline__ void column_chunk_any(const uint32_t* sw, int W, int count, int lane, const int2* sX,
                                              long long* a2) {
    long long alo = 0, ahi = 0;
    for (int e = 0; e < 32; ++e) {
        const int pos = e * W, wi = pos >> 5, off = pos & 31;
        const uint32_t lo = sw[wi * count + lane];
        const uint32_t hi = off + W > 32 ? sw[(wi + 1) * count + lane] : 0u;
        const uint32_t r = __funnelshift_r(lo, hi, off);
        const int c = W == 32 ? int(r) : (int(r << (32 - W)) >> (32 - W));
        const int2 xx = sX[e];
        alo += (long long)c * xx.x;
        ahi += (long long)c * xx.y;
    }
    a2[0] = alo;
    a2[1] = ahi;
}

// Descriptor fields of one column unit, kept one per lane.
struct ColDesc {
    long long word0;
    int col0, n, width, count, stride, comp_idx, chunk0, nchunks, part, nparts, split_id;
};

__device__ __forceinline__ ColDesc shfl_desc(const ColDesc& d, int src) {
    ColDesc r;
    r.word0 = __shfl_sync(0xFFFFFFFFu, d.word0, src);
    r.col0 = __shfl_sync(0xFFFFFFFFu, d.col0, src);
    r.n = __shfl_sync(0xFFFFFFFFu, d.n, src);
    r.width = __shfl_sync(0xFFFFFFFFu, d.width, src);
    r.count = __shfl_sync(0xFFFFFFFFu, d.count, src);
    r.stride = __shfl_sync(0xFFFFFFFFu, d.stride, src);
    r.comp_idx = __shfl_sync(0xFFFFFFFFu, d.comp_idx, src);
    r.chunk0 = __shfl_sync(0xFFFFFFFFu, d.chunk0, src);
    r.nchunks = __shfl_sync(0xFFFFFFFFu, d.nchunks, src);
    r.part = __shfl_sync(0xFFFFFFFFu, d.part, src);
    r.nparts = __shfl_sync(0xFFFFFFFFu, d.nparts, src);
    r.split_id = __shfl_sync(0xFFFFFFFFu, d.split_id, src);
    return r;
}

// Chunks of one (unit, column) that one pipeline step carries: as many as fit
// a slot (code words plus 32 x entries per chunk), at least one.
__device__ __forceinline__ int col_step_chunks(int stride, int remaining) {
    const int per = stride * 4 + kColChunk * 8;
    return max(1, min(remaining, (kSlotBytes - 16) / per));
}

// Column side.  Warp gw owns units gw, gw + G, ... (heaviest first); its work
// is the sequence (unit, rhs column, chunk), streamed through a kStages-deep
// pipeline of shared-memory slots filled by bulk copies (one per step for the
// code words, one for the x entries), kStages - 1 steps ahead of their use;
// a step carries as many chunks as fit a slot.  Lane l accumulates component
// l of the unit exactly; a unit's last chunk converts the sum (or, for a
// split task, hands it to the part that finishes last).
__global__ void __launch_bounds__(kWarps * 32, 2) column_kernel(Arena A, Work W, int n_tasks, int n, int rhs,
                                                                int n_comp, int max_parts, int* status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t s_bar[kWarps][kStages];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint8_t* slots = smem_raw + (size_t)warp * kStages * kSlotBytes;
    uint64_t* bar = s_bar[warp];
    if (lane == 0) {
        for (int i = 0; i < kStages; ++i) mbar_init(bar + i, 1);
        mbar_init_fence();
    }
    __syncwarp();
    const int G = gridDim.x * kWarps;
    const int gw = blockIdx.x * kWarps + warp;
    const int my_units = gw < n_tasks ? (n_tasks - gw + G - 1) / G : 0;
    unsigned issued = 0, computed = 0;  // running step counters (slot, phase)
    bool failed = false;
    for (int b0 = 0; b0 < my_units && !failed; b0 += 32) {
        const int nb = min(32, my_units - b0);
        ColDesc mine{};
        if (lane < nb) {
            const ColTask T = A.tasks[gw + (b0 + lane) * G];
            mine = {T.word0, T.col0, T.n, T.width, T.count, T.stride, T.comp_idx, T.chunk0, T.nchunks,
                    T.part, T.nparts, T.split_id};
        }
        int ik = 0, ip = 0, ic = 0;  // issue cursor
        ColDesc di = shfl_desc(mine, 0);
        auto issue = [&]() {
            if (ik >= nb) return;
            const int nc = col_step_chunks(di.stride, di.nchunks - ic);
            const unsigned slot_i = issued % kStages;
            uint8_t* slot = slots + slot_i * kSlotBytes;
            const unsigned wbytes = unsigned(nc * di.stride * 4);
            const int k0 = (di.chunk0 + ic) * kColChunk;
            const int cnt = min(di.n - k0, nc * kColChunk);
            const int2* xa = W.xl + (long long)ip * n + di.col0 + k0;
            const int xs = int((reinterpret_cast<uintptr_t>(xa) >> 3) & 1);
            const unsigned xbytes = unsigned(((cnt + xs) * 8 + 15) & ~15);
            if (lane == 0) {
                fence_async_smem();
                mbar_arrive_expect(bar + slot_i, wbytes + xbytes);
                bulk_load(slot, A.qwords + di.word0 + (long long)(di.chunk0 + ic) * di.stride, wbytes, bar + slot_i);
                bulk_load(slot + wbytes, xa - xs, xbytes, bar + slot_i);
            }
            ++issued;
            ic += nc;
            if (ic == di.nchunks) {
                ic = 0;
                if (++ip == rhs) {
                    ip = 0;
                    if (++ik < nb) di = shfl_desc(mine, ik);
                }
            }
        };
        __syncwarp();
#pragma unroll 1
        for (int s = 0; s < kStages - 1; ++s) issue();
        int ck = 0, cp = 0, cc = 0;  // compute cursor
        ColDesc dc = shfl_desc(mine, 0);
        __int128 acc = 0;
        int xe = W.xe[0];
        // finalize operands, loaded as soon as a unit starts
        int comp_id = lane < dc.count ? __ldg(A.task_comp + dc.comp_idx + lane) : 0;
        double comp_sc = lane < dc.count ? __ldg(A.comp_s + comp_id) : 0.0;
        while (ck < nb) {
            issue();
            const unsigned slot_i = computed % kStages;
            if (!mbar_wait(bar + slot_i, (computed / kStages) & 1)) {
                flag_timeout(status);
                failed = true;
                break;
            }
            const int nc = col_step_chunks(dc.stride, dc.nchunks - cc);
            const uint8_t* slot = slots + slot_i * kSlotBytes;
            const uint32_t* sw = reinterpret_cast<const uint32_t*>(slot);
            const int2* xa = W.xl + (long long)cp * n + dc.col0 + (dc.chunk0 + cc) * kColChunk;
            const int xs = int((reinterpret_cast<uintptr_t>(xa) >> 3) & 1);
            const int2* sxs = reinterpret_cast<const int2*>(slot + nc * dc.stride * 4) + xs;
            for (int c = 0; c < nc; ++c) {
                // x limbs of the chunk's entries (entries past the range meet
                // zero codes)
                const int2* sX = sxs + c * kColChunk;
                if (lane < dc.count) {
                    const uint32_t* cw = sw + c * dc.stride;
                    long long alo = 0, ahi = 0;
                    switch (dc.width) {
                        case 4: column_chunk<4>(cw, dc.count, lane, sX, alo, ahi); break;
                        case 8: column_chunk<8>(cw, dc.count, lane, sX, alo, ahi); break;
                        case 12: column_chunk<12>(cw, dc.count, lane, sX, alo, ahi); break;
                        case 16: column_chunk<16>(cw, dc.count, lane, sX, alo, ahi); break;
                        case 24: column_chunk<24>(cw, dc.count, lane, sX, alo, ahi); break;
                        case 32: column_chunk<32>(cw, dc.count, lane, sX, alo, ahi); break;
                        default: {
                            long long a2[2];
                            column_chunk_any(cw, dc.width, dc.count, lane, sX, a2);
                            alo = a2[0];
                            ahi = a2[1];
                        }
                    }
                    acc += widen(ahi, alo);
                }
            }
            ++computed;
            cc += nc;
            if (cc == dc.nchunks) {
                // finished (unit ck, column cp); x ~= X * 2^(xe - 1022 - kFixBits)
                if (dc.nparts == 1) {
                    if (lane < dc.count)
                        W.u[(long long)cp * n_comp + comp_id] = xe ? i128_ldexp(acc, xe - 1022 - kFixBits) * comp_sc : 0.0;
                } else {
                    long long* part = W.part + (((long long)dc.split_id * max_parts + dc.part) * rhs + cp) * 64;
                    part[2 * lane] = (long long)acc;
                    part[2 * lane + 1] = (long long)(acc >> 64);
                    __threadfence();
                    __syncwarp();
                    int done = 0;
                    if (lane == 0) done = atomicAdd(W.split_cnt + (long long)dc.split_id * rhs + cp, 1);
                    done = __shfl_sync(0xFFFFFFFFu, done, 0);
                    if (done == dc.nparts - 1) {
                        __threadfence();
                        __int128 tot = 0;
                        for (int q = 0; q < dc.nparts; ++q) {
                            const long long* pq =
                                W.part + (((long long)dc.split_id * max_parts + q) * rhs + cp) * 64;
                            const unsigned long long lo = __ldcg((const unsigned long long*)pq + 2 * lane);
                            const long long hi = __ldcg(pq + 2 * lane + 1);
                            tot += ((__int128)hi << 64) | lo;
                        }
                        if (lane < dc.count)
                            W.u[(long long)cp * n_comp + comp_id] =
                                xe ? i128_ldexp(tot, xe - 1022 - kFixBits) * comp_sc : 0.0;
                    }
                }
                acc = 0;
                cc = 0;
                if (++cp == rhs) {
                    cp = 0;
                    if (++ck < nb) {
                        dc = shfl_desc(mine, ck);
                        comp_id = lane < dc.count ? __ldg(A.task_comp + dc.comp_idx + lane) : 0;
                        comp_sc = lane < dc.count ? __ldg(A.comp_s + comp_id) : 0.0;
                    }
                }
                xe = W.xe[cp];
            }
            __syncwarp();
        }
    }
    // copies still in flight (only after a failed wait): wait for them, bounded
    while (computed < issued) {
        mbar_wait(bar + computed % kStages, (computed / kStages) & 1);
        ++computed;
    }
}

// acc (on exponent e_acc, kGuard guard bits) += v (on exponent ev); the
// accumulator's exponent rises to ev first if ev is larger.
__device__ __forceinline__ void add_aligned(__int128& acc0, __int128& acc1, int& e_acc, __int128 v0, __int128 v1,
                                            int ev) {
    if (ev > e_acc) {
        const int d = ev - e_acc;
        if (d >= 127) {
            acc0 = acc1 = 0;
        } else {
            const __int128 half = (__int128)1 << (d - 1);
            acc0 = (acc0 + half) >> d;
            acc1 = (acc1 + half) >> d;
        }
        e_acc = ev;
    }
    const int sh = (e_acc - ev) - kGuard;
    if (sh <= 0) {
        acc0 += v0 << (-sh);
        acc1 += v1 << (-sh);
    } else if (sh < 127) {
        const __int128 half = (__int128)1 << (sh - 1);
        acc0 += (v0 + half) >> sh;
        acc1 += (v1 + half) >> sh;
    }
}

struct RowDesc {
    int block, rloc0, comp, count, words;
    long long off;
};

// Row side: one CTA of kWarps warps per row tile; warp w owns the tile's
// units w, w + kWarps, ...; lane l owns tile rows 2l and 2l + 1.  Each warp
// streams its units (for every rhs column) through a kStages-deep cp.async
// pipeline (a unit's data block and its components' u values).  A unit's
// u are put in fixed point on the unit's own exponent, its row sums are exact,
// and they are added into 128-bit row accumulators kept on a running exponent
// with kGuard guard bits.  Dense diagonal units use FP64 loads directly.
// Warps combine per rhs column in shared memory in a fixed order.
__global__ void __launch_bounds__(kWarps * 32, 2) row_kernel(Arena A, Work W, double* __restrict__ y,
                                                             int n, int rhs, int n_comp, int* status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t s_bar[kWarps][kStages];
    __shared__ int s_e[kWarps];
    __shared__ double s_diag[kDenseSlices][kTileRows];
    __shared__ int s_nslices;
    __shared__ __align__(16) int4 s_tab[kWarps][32];
    const RowTile T = A.tiles[blockIdx.x];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint8_t* slots = smem_raw + (size_t)warp * kStages * kSlotBytes;
    uint64_t* bar = s_bar[warp];
    const int r0 = 2 * lane, r1 = 2 * lane + 1;
    const int nunits = T.item1 - T.item0;
    const int my = warp < nunits ? (nunits - warp + kWarps - 1) / kWarps : 0;
    if (threadIdx.x == 0) s_nslices = 0;
    if (lane == 0) {
        for (int i = 0; i < kStages; ++i) mbar_init(bar + i, 1);
        mbar_init_fence();
    }
    __syncthreads();
    unsigned issued = 0, computed = 0;  // running step counters (slot, phase)
    bool failed = false;
    // A warp's units, one descriptor per lane, in batches of 32; pipeline
    // steps carry as many consecutive units as fit a slot.
    for (int p = 0; p < rhs; ++p) {
        __int128 acc0 = 0, acc1 = 0;
        int e_acc = 0;
        for (int b0 = 0; b0 < my && !failed; b0 += 32) {
            const int nb = min(32, my - b0);
            RowDesc mine{};
            if (lane < nb) {
                const RowItem I = A.items[T.item0 + warp + (b0 + lane) * kWarps];
                mine = {I.block, I.rloc0, I.comp, I.count, I.words, I.off};
            }
            auto desc = [&](int k) {
                RowDesc d;
                d.block = __shfl_sync(0xFFFFFFFFu, mine.block, k);
                d.rloc0 = __shfl_sync(0xFFFFFFFFu, mine.rloc0, k);
                d.comp = __shfl_sync(0xFFFFFFFFu, mine.comp, k);
                d.count = __shfl_sync(0xFFFFFFFFu, mine.count, k);
                d.words = __shfl_sync(0xFFFFFFFFu, mine.words, k);
                d.off = __shfl_sync(0xFFFFFFFFu, mine.off, k);
                return d;
            };
            // bytes a unit occupies in a slot (words, then its u values copied
            // from an 8-byte-aligned start rounded down to 16 bytes)
            const int my_bytes =
                (lane < nb && mine.block >= 0) ? mine.words * 4 + ((mine.count + 1) * 8 + 15) / 16 * 16 : 0;
            auto group = [&](int k) {  // units [k, k + m) of one step
                int m = 1, tot = __shfl_sync(0xFFFFFFFFu, my_bytes, k);
                while (k + m < nb) {
                    const int b = __shfl_sync(0xFFFFFFFFu, my_bytes, k + m);
                    if (tot + b > kSlotBytes) break;
                    tot += b;
                    ++m;
                }
                return m;
            };
            int ik = 0;
            auto issue = [&]() {
                if (ik >= nb) return;
                const int m = group(ik);
                const unsigned slot_i = issued % kStages;
                uint8_t* slot = slots + slot_i * kSlotBytes;
                // total bytes of the step, then the copies (lane 0)
                unsigned total = 0;
                for (int q = 0; q < m; ++q) total += unsigned(__shfl_sync(0xFFFFFFFFu, my_bytes, ik + q));
                if (lane == 0) {
                    fence_async_smem();
                    mbar_arrive_expect(bar + slot_i, total);
                }
                int off = 0;
                for (int q = 0; q < m; ++q) {
                    const RowDesc d = desc(ik + q);
                    if (d.block < 0) continue;
                    const double* ua = W.u + (long long)p * n_comp + d.comp;
                    const int us = int((reinterpret_cast<uintptr_t>(ua) >> 3) & 1);
                    const unsigned ubytes = unsigned(((d.count + 1) * 8 + 15) / 16 * 16);
                    if (lane == 0) {
                        bulk_load(slot + off, A.pwords + d.off, unsigned(d.words * 4), bar + slot_i);
                        bulk_load(slot + off + d.words * 4, ua - us, ubytes, bar + slot_i);
                    }
                    off += d.words * 4 + int(ubytes);
                }
                ++issued;
                ik += m;
            };
            __syncwarp();
#pragma unroll 1
            for (int s = 0; s < kStages - 1; ++s) issue();
            int k = 0;
            while (k < nb) {
                issue();
                const unsigned slot_i = computed % kStages;
                if (!mbar_wait(bar + slot_i, (computed / kStages) & 1)) {
                    flag_timeout(status);
                    failed = true;
                    break;
                }
                const int m = group(k);
                const uint8_t* slot = slots + slot_i * kSlotBytes;
                int off = 0;
                for (int q = 0; q < m; ++q) {
                    const RowDesc d = desc(k + q);
                    if (d.block >= 0) {
                        const uint32_t* SW = reinterpret_cast<const uint32_t*>(slot + off);
                        const double* ua = W.u + (long long)p * n_comp + d.comp;
                        const int us = int((reinterpret_cast<uintptr_t>(ua) >> 3) & 1);
                        const double* SV = reinterpret_cast<const double*>(slot + off + d.words * 4) + us;
                        off += d.words * 4 + ((d.count + 1) * 8 + 15) / 16 * 16;
                        // widths from the header, u from the slot
                        int hw = 0;
                        double uv = 0.0;
                        if (lane < d.count) {
                            hw = int((SW[lane >> 1] >> (16 * (lane & 1))) & 0xFFFFu);
                            uv = SV[lane];
                        }
                        const int eb = __reduce_max_sync(0xFFFFFFFFu, lane < d.count ? exp_field(uv) : 0);
                        if (eb) {
                            const long long U = lane < d.count ? to_fixed(uv, eb) : 0;
                            int4* tab = s_tab[warp];
                            tab[lane] = make_int4(int(U & kLimbMask), int(U >> kLimb), hw >> 5, (hw & 31) + 1);
                            __syncwarp();
                            long long alo0 = 0, ahi0 = 0, alo1 = 0, ahi1 = 0;
                            long long blo0 = 0, bhi0 = 0, blo1 = 0, bhi1 = 0;
                            if (r0 < T.rows) {
                                int j = 0;
                                for (; j + 1 < d.count; j += 2) {
                                    const int4 t0 = tab[j], t1 = tab[j + 1];
                                    int c0, c1, e0, e1;
                                    row_pair_codes_rt(SW + t0.z, lane, t0.w, c0, c1);
                                    row_pair_codes_rt(SW + t1.z, lane, t1.w, e0, e1);
                                    alo0 += (long long)c0 * t0.x;
                                    ahi0 += (long long)c0 * t0.y;
                                    alo1 += (long long)c1 * t0.x;
                                    ahi1 += (long long)c1 * t0.y;
                                    blo0 += (long long)e0 * t1.x;
                                    bhi0 += (long long)e0 * t1.y;
                                    blo1 += (long long)e1 * t1.x;
                                    bhi1 += (long long)e1 * t1.y;
                                }
                                if (j < d.count) {
                                    const int4 t0 = tab[j];
                                    int c0, c1;
                                    row_pair_codes_rt(SW + t0.z, lane, t0.w, c0, c1);
                                    alo0 += (long long)c0 * t0.x;
                                    ahi0 += (long long)c0 * t0.y;
                                    alo1 += (long long)c1 * t0.x;
                                    ahi1 += (long long)c1 * t0.y;
                                }
                            }
                            alo0 += blo0;
                            ahi0 += bhi0;
                            alo1 += blo1;
                            ahi1 += bhi1;
                            __syncwarp();
                            __int128 v0 = widen(ahi0, alo0), v1 = widen(ahi1, alo1);
                            if (r0 >= T.rows) v0 = 0;
                            if (r1 >= T.rows) v1 = 0;
                            add_aligned(acc0, acc1, e_acc, v0, v1, eb);
                        }
                    } else {
                        // column slice of a dense diagonal block (column-major values)
                        const DenseDesc dd = A.dd[-1 - d.block];
                        const double* D = A.dense + d.off;
                        const double* xcp = W.xc + (long long)p * n + dd.col0 + d.words;
                        double dg0 = 0.0, dg1 = 0.0;
                        const bool v0 = r0 < T.rows, v1 = r1 < T.rows;
                        // eight columns at a time: all loads issued before the FMA chain
                        for (int k0 = 0; k0 < d.count; k0 += 8) {
                            double xv[8], a0v[8], a1v[8];
#pragma unroll
                            for (int q = 0; q < 8; ++q) {
                                const int kk = k0 + q;
                                const bool in = kk < d.count;
                                const double* col = D + (long long)kk * dd.m;
                                xv[q] = in ? __ldg(xcp + kk) : 0.0;
                                a0v[q] = (in && v0) ? __ldg(col + r0) : 0.0;
                                a1v[q] = (in && v1) ? __ldg(col + r1) : 0.0;
                            }
#pragma unroll
                            for (int q = 0; q < 8; ++q) {
                                dg0 = fma(a0v[q], xv[q], dg0);
                                dg1 = fma(a1v[q], xv[q], dg1);
                            }
                        }
                        s_diag[d.comp][r0] = dg0;
                        s_diag[d.comp][r1] = dg1;
                        if (lane == 0) atomicMax(&s_nslices, d.comp + 1);
                    }
                }
                k += m;
                ++computed;
                __syncwarp();
            }
            // after a failed wait the warp does no more work but still takes
            // part in the tile's barriers below
        }
        // row sums go to the warp's own (drained) stage 0 for the combine
        __int128* wacc = reinterpret_cast<__int128*>(slots);
        wacc[r0] = acc0;
        wacc[r1] = acc1;
        if (lane == 0) s_e[warp] = e_acc;
        __syncthreads();
        if (threadIdx.x < T.rows) {
            const int r = threadIdx.x;
            int et = 0;
#pragma unroll
            for (int i = 0; i < kWarps; ++i) et = max(et, s_e[i]);
            __int128 tot = 0;
#pragma unroll
            for (int i = 0; i < kWarps; ++i) {
                const int dsh = et - s_e[i];
                const __int128 a = reinterpret_cast<const __int128*>(smem_raw + (size_t)i * kStages * kSlotBytes)[r];
                if (dsh == 0) tot += a;
                else if (dsh < 127) tot += (a + ((__int128)1 << (dsh - 1))) >> dsh;
            }
            const double lr = et ? i128_ldexp(tot, et - 1022 - kFixBits - kGuard) : 0.0;
            double dg = 0.0;
            for (int sl = 0; sl < s_nslices; ++sl) dg += s_diag[sl][r];
            y[(long long)__ldg(A.perm + T.row0 + r) * rhs + p] = dg + lr;
        }
        __syncthreads();
    }
    // copies still in flight (only after a failed wait): wait for them, bounded
    while (computed < issued) {
        mbar_wait(bar + computed % kStages, (computed / kStages) & 1);
        ++computed;
    }
}

// Validation: decode every code through the same device routines the apply
// kernels use (code_at / row_pair_codes on the resident layout).  Column
// side: one warp per unit; row side: one warp per tile.
template <int W>
__device__ __forceinline__ void col_codes(const uint32_t* cw, int count, int lane, int (&c)[32]) {
    uint32_t w[W];
#pragma unroll
    for (int v = 0; v < W; ++v) w[v] = cw[v * count + lane];
#pragma unroll
    for (int e = 0; e < 32; ++e) c[e] = code_at<W>(w, e);
}

__global__ void decode_col_kernel(Arena A, int n_tasks, const long long* __restrict__ comp_off, int* out) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int ti = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ti < n_tasks; ti += warps) {
        const ColTask T = A.tasks[ti];
        if (lane >= T.count) continue;
        const long long o = comp_off[__ldg(A.task_comp + T.comp_idx + lane)];
        for (int ch = T.chunk0; ch < T.chunk0 + T.nchunks; ++ch) {
            const uint32_t* cw = A.qwords + T.word0 + (long long)ch * T.stride;
            int c[32];
            switch (T.width) {
#define QH_DEC_CASE(WW) \
    case WW:            \
        col_codes<WW>(cw, T.count, lane, c); \
        break;
                QH_WIDTH_CASES(QH_DEC_CASE)
#undef QH_DEC_CASE
                default:
                    break;
            }
            for (int e = 0; e < 32; ++e)
                if (ch * kColChunk + e < T.n) out[o + ch * kColChunk + e] = c[e];
        }
    }
}

__global__ void decode_row_kernel(Arena A, int n_tiles, const long long* __restrict__ comp_off, int* out) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < n_tiles; t += warps) {
        const RowTile T = A.tiles[t];
        for (int it = T.item0; it < T.item1; ++it) {
            const RowItem I = A.items[it];
            if (I.block < 0) continue;
            const uint32_t* blk = A.pwords + I.off;
            for (int j = 0; j < I.count; ++j) {
                const int hw = int((blk[j >> 1] >> (16 * (j & 1))) & 0xFFFFu);
                const int w = (hw & 31) + 1;
                const uint32_t* piece = blk + (hw >> 5);
                int c0 = 0, c1 = 0;
                if (2 * lane < T.rows) row_pair_codes_rt(piece, lane, w, c0, c1);
                const long long o = comp_off[I.comp + j] + I.rloc0;
                if (2 * lane < T.rows) out[o + 2 * lane] = c0;
                if (2 * lane + 1 < T.rows) out[o + 2 * lane + 1] = c1;
            }
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

// Scratch of qh_matmul_device_static: one fixed array per device, loaded with
// the library and held until exit.  Host code must not use this symbol as an
// address (it names a host-side stand-in); static_scratch() returns the
// device address for the current device.
static __device__ __align__(256) unsigned char g_static_scratch[QH_STATIC_SCRATCH_BYTES];

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
    e = cudaFuncSetAttribute(row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPipeSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(column_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPipeSmem);
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "cudaFuncSetAttribute");
    }
    // The host image is no longer needed once uploaded.
    std::vector<uint8_t>().swap(m->L.arena);
    const Sections& S = m->L.sec;
    auto* base = static_cast<const uint8_t*>(m->arena);
    m->A.perm = reinterpret_cast<const int32_t*>(base + S.perm);
    m->A.lr = reinterpret_cast<const LowRankDesc*>(base + S.lr);
    m->A.dd = reinterpret_cast<const DenseDesc*>(base + S.dd);
    m->A.comp_w = base + S.comp_w;
    m->A.comp_s = reinterpret_cast<const double*>(base + S.comp_s);
    m->A.tasks = reinterpret_cast<const ColTask*>(base + S.tasks);
    m->A.task_comp = reinterpret_cast<const int32_t*>(base + S.task_comp);
    m->A.qwords = reinterpret_cast<const uint32_t*>(base + S.qwords);
    m->A.pwords = reinterpret_cast<const uint32_t*>(base + S.pwords);
    m->A.dense = reinterpret_cast<const double*>(base + S.dense);
    m->A.tiles = reinterpret_cast<const RowTile*>(base + S.tiles);
    m->A.items = reinterpret_cast<const RowItem*>(base + S.items);
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
    size_t xc, xl, xe, cnt, part, u, total, zero_bytes;
};

WsPlan ws_plan(const Layout& L, size_t rhs) {
    WsPlan w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += align256(std::max<size_t>(bytes, 1));
        return o;
    };
    // zeroed before each apply: xe and the split counters (contiguous)
    w.xe = take(4 * rhs);
    w.cnt = take(4 * size_t(L.n_split) * rhs);
    w.zero_bytes = off;
    // xc and u are read by 16-byte-rounded bulk copies: keep 32 spare bytes
    w.xc = take(8 * L.order * rhs + 32);
    w.xl = take(8 * L.order * rhs + 32);
    w.part = take(16 * 32 * size_t(L.n_split) * size_t(L.max_parts) * rhs);
    w.u = take(8 * size_t(L.n_comp) * rhs + 32);
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
    W.xc = reinterpret_cast<double*>(w + P.xc);
    W.xl = reinterpret_cast<int2*>(w + P.xl);
    W.xe = reinterpret_cast<int*>(w + P.xe);
    W.split_cnt = reinterpret_cast<int*>(w + P.cnt);
    W.part = reinterpret_cast<long long*>(w + P.part);
    W.u = reinterpret_cast<double*>(w + P.u);
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[i]), s);
    };
    const long long prep_warps = (long long)L.n_chunks * (long long)rhs;
    mark(0);
    cudaError_t e = cudaMemsetAsync(w, 0, P.zero_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    prep_x_kernel<<<unsigned((prep_warps + 7) / 8), 256, 0, s>>>(m->A, W, x, n, int(rhs), L.n_chunks, status);
    x_limbs_kernel<<<unsigned(((long long)n * (long long)rhs + 255) / 256), 256, 0, s>>>(W, n, int(rhs));
    mark(1);
    if (L.n_tasks > 0) {
        const int grid = std::max(1, std::min((L.n_tasks + kWarps - 1) / kWarps, m->sms * 2));
        column_kernel<<<grid, kWarps * 32, kPipeSmem, s>>>(m->A, W, L.n_tasks, n, int(rhs), L.n_comp, L.max_parts,
                                                            status);
    }
    mark(2);
    row_kernel<<<L.n_tiles, kWarps * 32, kPipeSmem, s>>>(m->A, W, y, n, int(rhs), L.n_comp, status);
    mark(3);
    e = cudaGetLastError();
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

int qh_matmul_device_static(const qh_matrix* m, const double* x, double* y, size_t rhs, void* stream,
                            int* status) {
    if (!m) return fail(QH_EINVAL, "null matrix handle");
    int rc = check_rhs(m, rhs);
    if (rc) return rc;
    if (!x || !y) return fail(QH_EINVAL, "null right-hand side or result pointer");
    const size_t need = ws_bytes(m->L, rhs);
    if (need > size_t(QH_STATIC_SCRATCH_BYTES))
        return fail(QH_EINVAL, "qh_matmul_device_static: this apply needs " + std::to_string(need) +
                                   " bytes of scratch, more than the fixed " +
                                   std::to_string(size_t(QH_STATIC_SCRATCH_BYTES)) +
                                   " (QH_STATIC_SCRATCH_BYTES); use qh_matmul_device with a workspace");
    DeviceGuard g(m->device);
    // Device address of the array, looked up once per device with that device
    // current (the first call on a device does this set-up).
    static std::mutex mu;
    static void* addr[64] = {nullptr};
    if (m->device < 0 || m->device >= 64) return fail(QH_EINVAL, "invalid CUDA device ordinal");
    void* ptr = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!addr[m->device]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
            addr[m->device] = p;
        }
        ptr = addr[m->device];
    }
    return launch(m, x, y, rhs, ptr, static_cast<cudaStream_t>(stream), status);
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
    if (*mm->h_status & kStatusNonfinite) return fail(QH_EINVAL, "nonfinite right-hand side");
    if (*mm->h_status & kStatusTimeout) return fail(QH_ERUNTIME, "device copy wait timed out");
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
        // component-major output: component c's codes start at off[c]
        std::vector<long long> off(size_t(m->L.n_comp) + 1, 0);
        for (const auto& d : lr)
            for (int j = 0; j < d.rank; ++j)
                off[size_t(d.comp0 + j) + 1] = side == 0 ? d.m : d.n;
        for (size_t c = 0; c + 1 < off.size(); ++c) off[c + 1] += off[c];
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
            if (side == 1)
                decode_col_kernel<<<std::max(1, std::min((m->L.n_tasks + 7) / 8, 4096)), 256>>>(m->A, m->L.n_tasks, d_off, d_out);
            else
                decode_row_kernel<<<std::max(1, std::min((m->L.n_tiles + 7) / 8, 4096)), 256>>>(m->A, m->L.n_tiles, d_off, d_out);
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
