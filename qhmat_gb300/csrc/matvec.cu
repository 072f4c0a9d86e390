// GB300 (sm_103a) resident quantized H-matrix matvec and its C ABI.
//
// y = A x for a matrix held as dense FP64 diagonal blocks plus low-rank blocks
// whose balanced factors P (rows) and Q (columns) are stored as per-component
// signed integer codes of width w_j in [2, 32] (src/qhmat/core.cpp:235-282),
// with one FP64 scale per factor and component.  The resident layout
// (layout.hpp) keeps each code's bits, re-ordered into tensor-core fragment
// order as base-256 digit planes.
//
// FP64 throughput on GB300 is a small fraction of its tensor throughput, so
// every code product is an exact small-integer product on the f16 tensor
// cores (digits <= 255 times 8-bit limbs of a fixed-point operand, FP32 sums
// that stay integers below 2^24), and FP64 is used only per component, per
// output row and for the dense diagonal blocks:
//
//   prep_x / x_limbs   x (source order) -> clustered order; one exponent per
//                      rhs column; X = round(x 2^(62-e)) as eight f16 limbs.
//   column_kernel      warp per task (<= 32 components sharing a column range
//                      and a width): t_j = sum_i c_ij X_i exactly, then
//                      u_j = (s^P s^Q) t_j 2^(e-1022-62) in FP64, then u in
//                      fixed point on each consuming row tile's exponent (a
//                      layout-time bound) as that tile's B rows (limbs);
//                      and warp per dense unit (16 columns of a dense
//                      diagonal block part, FP64 row sums).
//   row_kernel         warp per (row tile, 16 rows, k split): sum_j c_ij U_j
//                      exactly, stored as 128-bit partial sums.
//   combine_kernel     thread per row: dense row sums in column order plus
//                      the partials -> y (one conversion).
//
// The only rounding steps are the fixed-point conversions of x and u (2^-63
// of the column's largest |x|, of the tile's bound on |u|), the product
// s^P s^Q, and the final FP64 conversions: the result agrees with the
// reference's FP64 matmul (src/qhmat/core.cpp:360-390) to ~1e-15 in norm.
#include <cooperative_groups.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <queue>
#include <type_traits>
#include <string>
#include <vector>

#include <unistd.h>

#include "../../include/qhmat_gb300.h"
#include "batch.hpp"
#include "errors.hpp"
#include "layout.hpp"

namespace qhg {
namespace {

// Fixed point: x (per rhs column) and u (per row tile) are held as integers
// X = round(v * 2^(kFixBits - (e - 1022))), |X| <= 2^kFixBits, on one exponent
// field e; the tensor-core operand is X's eight base-256 limbs (seven unsigned,
// the top one signed), each an exact f16.
constexpr int kFixBits = 62;


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

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}
__device__ __forceinline__ uint32_t hsub2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("sub.f16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

// The eight limbs of X (|X| <= 2^62) as f16 values, limb k in half k:
// X = sum_{k<7} l_k 2^(8k) + l_7 2^56 with l_0..l_6 in [0, 255] and l_7 in
// [-64, 64].  The bytes of X + 2^62 are those limbs, the top one plus 64;
// byte b becomes the f16 1024 + b (exponent bits 0x64 above it) and then the
// integer b by one exact subtraction per pair.
__device__ __forceinline__ uint4 to_limbs(long long X) {
    const unsigned long long Y = (unsigned long long)X + (1ull << 62);
    const uint32_t lo = uint32_t(Y), hi = uint32_t(Y >> 32);
    return make_uint4(hsub2(prmt(lo, 0x64646464u, 0x4140u), 0x64006400u),
                      hsub2(prmt(lo, 0x64646464u, 0x4342u), 0x64006400u),
                      hsub2(prmt(hi, 0x64646464u, 0x4140u), 0x64006400u),
                      hsub2(prmt(hi, 0x64646464u, 0x4342u), 0x64406400u));
}

struct Arena {
    const int32_t* perm;   // clustered position -> source index
    const int32_t* iperm;  // source index -> clustered position
    const LowRankDesc* lr;
    const DenseDesc* dd;
    const uint8_t* comp_w;
    const double* comp_s;
    const ColTask* tasks;
    const TaskRec* task_rec;
    const uint8_t* qcodes;
    const uint8_t* pcodes;
    const double* dense;
    const RowTile* tiles;
    const TileDense* tdense;
    const RowUnit* units;
    const uint8_t* kp_info;
    const SlotRec* slot_rec;
    const TaskDest* task_dest;
    const uint32_t* row_steps;
    const double* comp_sl;  // s^P per component
    const double* comp_sr;  // s^Q per component
};

struct Work {
    double* xc;        // [rhs][n]            x in clustered order (FP64)
    int* xblk;         // [rhs][nblk]         largest exponent field of x per prep block
    int* xe;           // [rhs]               largest exponent field of x
    uint4* xq;         // [rhs][n_pad]        limbs of X (zero past n)
    long long* lsplit; // [rhs][n_split*33][8] per-limb sums sum_i c_ij limb_l(X_i) of split tasks'
                       //                     components (rows split_id*33 + j; zeroed by prep)
    int* split_cnt;    // [rhs][n_split]      finished parts of each split task (zeroed by prep)
    uint4* blimb;      // [rhs][n_slots]      row-side B rows: limbs of U
    uint4* plr;        // [rhs][n_tiles][kTileUnits][16] low-rank row sums of each row unit (128-bit)
    double* pdense;    // [rhs][n_dslices][64] dense diagonal row sums per dense slice
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
// Potentially blocking test of a phase: the thread waits until the phase
// completes or a system-dependent time limit passes (measured faster than an
// explicit suspend-time hint, which delays the wake-up).
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up (returns false) after `limit` tests (kWaitLimit:
// seconds at most) instead of hanging; callers record the failure in the
// status word, stop issuing copies, give the copies already issued one more
// bounded wait each and return (best effort: a copy still outstanding after
// that wait is abandoned with the block).
constexpr int kWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int limit = kWaitLimit) {
    for (int i = 0; i < limit; ++i)
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

// Programmatic dependent launch: a kernel lets its successor start early
// (launch_dependents) and waits for its predecessor's results (wait) only
// where it first reads them; without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Pipeline depth and CTAs per SM of the two streaming kernels (measured:
// two stages per warp and two CTAs of 8 warps per SM; capping registers for a
// third CTA spills the accumulators).
#ifndef QH_COL_STAGES
#define QH_COL_STAGES 2
#define QH_COL_CTAS 2
#endif
#ifndef QH_ROW_STAGES
#define QH_ROW_STAGES 2
#define QH_ROW_CTAS 2
#endif
constexpr int kColStages = QH_COL_STAGES;
constexpr int kRowStages = QH_ROW_STAGES;
constexpr int kWarps = 8;
constexpr int kColPipeSmem = kWarps * kColStages * kColSlotBytes;
// Unit descriptors a column warp keeps in shared memory.
constexpr int kStagedUnits = 24;
constexpr int kRowPipeSmem = kWarps * kRowStages * kRowSlotBytes;

// Status bits written by the kernels (status word of the apply).
constexpr int kStatusNonfinite = QH_STATUS_NONFINITE;
constexpr int kStatusTimeout = QH_STATUS_TIMEOUT;

__device__ __forceinline__ void flag_timeout(int* status) {
    if (status) atomicOr(status, kStatusTimeout);
}

// Test aid for the bounded wait: one warp waits, `polls` tests at most, on an
// mbarrier that nothing ever completes (no copy is issued, so giving up
// leaves nothing in flight) and records the timeout in the status word
// exactly as the streaming kernels do.
__global__ void wait_timeout_kernel(int polls, int* status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncwarp();
    const bool ok = mbar_wait(&bar, 0, polls);
    if (!ok && threadIdx.x == 0) flag_timeout(status);
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

__device__ __forceinline__ __int128 shfl_xor_i128(__int128 v, int m) {
    const long long lo = __shfl_xor_sync(0xFFFFFFFFu, (long long)v, m);
    const long long hi = __shfl_xor_sync(0xFFFFFFFFu, (long long)(v >> 64), m);
    return ((__int128)hi << 64) | (unsigned long long)lo;
}

// ------------------------------------------------- tensor-core fragments
//
// A digit d enters the MMA as the f16 bit pattern d, i.e. the subnormal
// d * 2^-24, so a byte or nibble becomes an operand with one permute (bytes)
// or one shift-and-mask (nibbles); products with the normal-f16 limbs are
// exact and every accumulator value is an integer times 2^-24 below 1, exact
// in FP32.

// Byte group word (digits of entries 2t, 2t+1, 2t+8, 2t+9): the f16 pairs of
// entries (2t, 2t+1) and (2t+8, 2t+9).
__device__ __forceinline__ uint32_t dig_lo(uint32_t w) { return prmt(w, 0u, 0x4140u); }
__device__ __forceinline__ uint32_t dig_hi(uint32_t w) { return prmt(w, 0u, 0x4342u); }
// Nibble group word: pair k = (nibble k, nibble k + 4); k = 0, 1 are k-block
// 0's pairs (2t, 2t+1) and (2t+8, 2t+9), k = 2, 3 k-block 1's.
__device__ __forceinline__ uint32_t nib_pair(uint32_t v, int k) { return (v >> (4 * k)) & 0x000F000Fu; }

// d += A * B for one 16x8x16 step (A: rows g, g+8 x k 2t.., 2t+8..).
__device__ __forceinline__ void mma_dig(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                        uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// B fragments of two k-blocks from 32 rows of 16 bytes (limbs of 32 entries
// or components) at a 16-byte-aligned shared address: lane l points at row l.
__device__ __forceinline__ void limb_frags(uint32_t row_addr, uint32_t (&b)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
                 : "r"(row_addr)
                 : "memory");
}

// One group (rows g and g+8 of a 16-row fragment pair of k-blocks, in
// shared memory at grp) into d.  Byte rows are 32 bytes, nibble rows 16; rows
// >= `rows` are zero.  Plain loads (ordered after the stage's mbarrier wait,
// which clobbers memory) and non-volatile MMAs leave the compiler free to
// overlap one group's loads with the previous group's MMAs.
__device__ __forceinline__ void group_mma(float (&d)[4], const uint8_t* grp, bool nib, int rows, int g, int t,
                                          const uint32_t (&b)[4]) {
    if (nib) {
        const uint32_t v0 = g < rows ? *reinterpret_cast<const uint32_t*>(grp + g * 16 + 4 * t) : 0u;
        const uint32_t v1 = g + 8 < rows ? *reinterpret_cast<const uint32_t*>(grp + (g + 8) * 16 + 4 * t) : 0u;
        mma_dig(d, nib_pair(v0, 0), nib_pair(v1, 0), nib_pair(v0, 1), nib_pair(v1, 1), b[0], b[1]);
        mma_dig(d, nib_pair(v0, 2), nib_pair(v1, 2), nib_pair(v0, 3), nib_pair(v1, 3), b[2], b[3]);
    } else {
        const uint2 w0 = g < rows ? *reinterpret_cast<const uint2*>(grp + g * 32 + 8 * t) : make_uint2(0u, 0u);
        const uint2 w1 =
            g + 8 < rows ? *reinterpret_cast<const uint2*>(grp + (g + 8) * 32 + 8 * t) : make_uint2(0u, 0u);
        mma_dig(d, dig_lo(w0.x), dig_lo(w1.x), dig_hi(w0.x), dig_hi(w1.x), b[0], b[1]);
        mma_dig(d, dig_lo(w0.y), dig_lo(w1.y), dig_hi(w0.y), dig_hi(w1.y), b[2], b[3]);
    }
}

// The top plane of a column task: stored digits s = d + 2^(t-1) become the
// signed digit d as a normal f16 (1024 + s, minus hb = 1024 + 2^(t-1) in both
// halves), so no offset correction is needed on the column side.
__device__ __forceinline__ uint32_t top_lo(uint32_t w, uint32_t hb) { return hsub2(prmt(w, 0x64646464u, 0x4140u), hb); }
__device__ __forceinline__ uint32_t top_hi(uint32_t w, uint32_t hb) { return hsub2(prmt(w, 0x64646464u, 0x4342u), hb); }
__device__ __forceinline__ uint32_t top_nib(uint32_t v, int k, uint32_t hb) {
    return hsub2(nib_pair(v, k) | 0x64006400u, hb);
}
__device__ __forceinline__ void group_mma_top(float (&d)[4], const uint8_t* grp, bool nib, int rows, int g, int t,
                                              const uint32_t (&b)[4], uint32_t hb) {
    // rows past `rows` contribute zero: their operands are forced to +0.0
    const bool in0 = g < rows, in1 = g + 8 < rows;
    if (nib) {
        const uint32_t v0 = in0 ? *reinterpret_cast<const uint32_t*>(grp + g * 16 + 4 * t) : 0u;
        const uint32_t v1 = in1 ? *reinterpret_cast<const uint32_t*>(grp + (g + 8) * 16 + 4 * t) : 0u;
        uint32_t a[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            a[k] = in0 ? top_nib(v0, k, hb) : 0u;
            a[4 + k] = in1 ? top_nib(v1, k, hb) : 0u;
        }
        mma_dig(d, a[0], a[4], a[1], a[5], b[0], b[1]);
        mma_dig(d, a[2], a[6], a[3], a[7], b[2], b[3]);
    } else {
        const uint2 w0 = in0 ? *reinterpret_cast<const uint2*>(grp + g * 32 + 8 * t) : make_uint2(0u, 0u);
        const uint2 w1 = in1 ? *reinterpret_cast<const uint2*>(grp + (g + 8) * 32 + 8 * t) : make_uint2(0u, 0u);
        const uint32_t a0 = in0 ? top_lo(w0.x, hb) : 0u, a2 = in0 ? top_hi(w0.x, hb) : 0u;
        const uint32_t a4 = in0 ? top_lo(w0.y, hb) : 0u, a6 = in0 ? top_hi(w0.y, hb) : 0u;
        const uint32_t a1 = in1 ? top_lo(w1.x, hb) : 0u, a3 = in1 ? top_hi(w1.x, hb) : 0u;
        const uint32_t a5 = in1 ? top_lo(w1.y, hb) : 0u, a7 = in1 ? top_hi(w1.y, hb) : 0u;
        mma_dig(d, a0, a1, a2, a3, b[0], b[1]);
        mma_dig(d, a4, a5, a6, a7, b[2], b[3]);
    }
}

// The top plane of a row k-pair: stored digits s = d + 2^(t-1) become the
// signed digit d on the lower planes' scale, d 2^-24 (a subnormal f16 for
// |d| < 1024): the f16 with exponent field 1 and mantissa s is (1024 + s)
// 2^-24, minus hb = (1024 + 2^(t-1)) 2^-24 in both halves, exactly.
__device__ __forceinline__ uint32_t rtop_lo(uint32_t w, uint32_t hb) { return hsub2(prmt(w, 0x04040404u, 0x4140u), hb); }
__device__ __forceinline__ uint32_t rtop_hi(uint32_t w, uint32_t hb) { return hsub2(prmt(w, 0x04040404u, 0x4342u), hb); }
__device__ __forceinline__ uint32_t rtop_nib(uint32_t v, int k, uint32_t hb) {
    return hsub2(nib_pair(v, k) | 0x04000400u, hb);
}
__device__ __forceinline__ void group_mma_rtop(float (&d)[4], const uint8_t* grp, bool nib, int g, int t,
                                               const uint32_t (&b)[4], uint32_t hb) {
    if (nib) {
        const uint32_t v0 = *reinterpret_cast<const uint32_t*>(grp + g * 16 + 4 * t);
        const uint32_t v1 = *reinterpret_cast<const uint32_t*>(grp + (g + 8) * 16 + 4 * t);
        mma_dig(d, rtop_nib(v0, 0, hb), rtop_nib(v1, 0, hb), rtop_nib(v0, 1, hb), rtop_nib(v1, 1, hb), b[0], b[1]);
        mma_dig(d, rtop_nib(v0, 2, hb), rtop_nib(v1, 2, hb), rtop_nib(v0, 3, hb), rtop_nib(v1, 3, hb), b[2], b[3]);
    } else {
        const uint2 w0 = *reinterpret_cast<const uint2*>(grp + g * 32 + 8 * t);
        const uint2 w1 = *reinterpret_cast<const uint2*>(grp + (g + 8) * 32 + 8 * t);
        mma_dig(d, rtop_lo(w0.x, hb), rtop_lo(w1.x, hb), rtop_hi(w0.x, hb), rtop_hi(w1.x, hb), b[0], b[1]);
        mma_dig(d, rtop_lo(w0.y, hb), rtop_lo(w1.y, hb), rtop_hi(w0.y, hb), rtop_hi(w1.y, hb), b[2], b[3]);
    }
}

// Digits of rows g, g+8 of a group as integers, in the order the MMA sees
// them (for validation): out[half][kb*4 + s], s = entries 2t, 2t+1, 2t+8, 2t+9.
__device__ __forceinline__ void group_digits(const uint8_t* grp, bool nib, int rows, int g, int t,
                                             uint32_t (&out)[2][8]) {
    uint32_t r[2][4];  // [half][kb0 lo, kb0 hi, kb1 lo, kb1 hi]
    if (nib) {
        const uint32_t v0 = g < rows ? *reinterpret_cast<const uint32_t*>(grp + g * 16 + 4 * t) : 0u;
        const uint32_t v1 = g + 8 < rows ? *reinterpret_cast<const uint32_t*>(grp + (g + 8) * 16 + 4 * t) : 0u;
        for (int k = 0; k < 4; ++k) {
            r[0][k] = nib_pair(v0, k);
            r[1][k] = nib_pair(v1, k);
        }
    } else {
        const uint2 w0 = g < rows ? *reinterpret_cast<const uint2*>(grp + g * 32 + 8 * t) : make_uint2(0u, 0u);
        const uint2 w1 =
            g + 8 < rows ? *reinterpret_cast<const uint2*>(grp + (g + 8) * 32 + 8 * t) : make_uint2(0u, 0u);
        r[0][0] = dig_lo(w0.x), r[0][1] = dig_hi(w0.x), r[0][2] = dig_lo(w0.y), r[0][3] = dig_hi(w0.y);
        r[1][0] = dig_lo(w1.x), r[1][1] = dig_hi(w1.x), r[1][2] = dig_lo(w1.y), r[1][3] = dig_hi(w1.y);
    }
    for (int hh = 0; hh < 2; ++hh)
        for (int k = 0; k < 4; ++k) {
            // pair k: k-block k >> 1, slots (2(k&1), 2(k&1) + 1)
            out[hh][(k >> 1) * 4 + 2 * (k & 1)] = r[hh][k] & 0xFFFFu;
            out[hh][(k >> 1) * 4 + 2 * (k & 1) + 1] = r[hh][k] >> 16;
        }
}
// Entry (within a 32-entry k-pair) of slot s of k-block kb for thread t.
__device__ __forceinline__ int slot_entry(int kb, int s, int t) { return 16 * kb + 2 * t + (s & 1) + 8 * (s >> 1); }

// Exact integers sum(D * 2^24) of a plane's accumulators, folded into 64-bit
// sums at weight 2^(8m).
__device__ __forceinline__ long long fold(float d, int m) {
    return (long long)__float2int_rn(d * 16777216.0f) << (8 * m);
}

// Widths a code may have (the reference's writer allows 2..32).
#define QH_WIDTH_CASES(X) \
    X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17) \
    X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31) X(32)

// ---------------------------------------------------------------- kernels

__device__ __forceinline__ void st_i128(uint4* p, __int128 v) {
    *p = make_uint4(uint32_t(v), uint32_t(v >> 32), uint32_t(v >> 64), uint32_t(v >> 96));
}
__device__ __forceinline__ __int128 ld_i128(const uint4* p) {
    const uint4 v = __ldcg(p);
    return (__int128)(((unsigned __int128)v.w << 96) | ((unsigned __int128)v.z << 64) |
                      ((unsigned __int128)v.y << 32) | v.x);
}

// Block (bx, p) of 8 warps: source entries 256bx .. 256bx+255 of rhs column
// p, read in order (coalesced; x may be the caller's host memory, read over
// the coherent host link) and stored at their clustered positions as the
// FP64 copy of x; the block's largest exponent field; nonfinite flag.  The
// grid also zeroes the apply's counters.
__device__ __forceinline__ void prep_block(const Arena& A, const Work& W, const double* __restrict__ x, int n,
                                           long long ld, int n_chunks, int* zero, int n_zero, int* status,
                                           int* s_m) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int p = blockIdx.y;
    const int chunk = blockIdx.x * 8 + warp;
    const int src = chunk * kChunk + lane;
    const bool valid = chunk < n_chunks && src < n;
    const double v = valid ? x[(long long)src * ld + p] : 0.0;  // (plain load)
    const int e = exp_field(v);
    if (__any_sync(0xFFFFFFFFu, e == 0x7FF) && lane == 0 && status) atomicOr(status, kStatusNonfinite);
    const int em = __reduce_max_sync(0xFFFFFFFFu, e == 0x7FF ? 0 : e);
    if (valid) W.xc[(long long)p * n + __ldg(A.iperm + src)] = e == 0x7FF ? 0.0 : v;
    if (lane == 0) s_m[warp] = em;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = 0;
        for (int i = 0; i < 8; ++i) m = max(m, s_m[i]);
        W.xblk[(long long)p * gridDim.x + blockIdx.x] = m;
    }
    const long long tid = ((long long)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
    const long long nthr = (long long)gridDim.x * gridDim.y * blockDim.x;
    for (long long i = tid; i < n_zero; i += nthr) zero[i] = 0;
}

__global__ void __launch_bounds__(256) prep_x_kernel(Arena A, Work W, const double* __restrict__ x, int n,
                                                     long long ld, int n_chunks, int* zero, int n_zero,
                                                     int* status) {
    __shared__ int s_m[8];
    pdl_trigger();
    prep_block(A, W, x, n, ld, n_chunks, zero, n_zero, status, s_m);
}

// Blocks bx = 0, nbx, ... of rhs column p: the column's exponent from the prep
// blocks' maxima, then the limbs of X for entries bx*256 .. (zero past n).
__device__ __forceinline__ void limbs_block(const Work& W, int n, int n_pad, int nblk, int p, int bx, int nbx,
                                            int* s_m) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int m = 0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) m = max(m, __ldcg(W.xblk + (long long)p * nblk + i));
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    __syncthreads();  // (s_m reused)
    if (lane == 0) s_m[warp] = m;
    __syncthreads();
    int xe = 0;
    for (int i = 0; i < 8; ++i) xe = max(xe, s_m[i]);
    if (bx == 0 && threadIdx.x == 0) W.xe[p] = xe;
    for (int k = bx * blockDim.x + threadIdx.x; k < n_pad; k += nbx * blockDim.x) {
        const long long X = (k < n && xe) ? to_fixed(__ldcg(W.xc + (long long)p * n + k), xe) : 0;
        W.xq[(long long)p * n_pad + k] = to_limbs(X);
    }
}

__global__ void __launch_bounds__(256) x_limbs_kernel(Work W, int n, int n_pad, int nblk) {
    __shared__ int s_m[8];
    pdl_trigger();
    pdl_wait();
    limbs_block(W, n, n_pad, nblk, blockIdx.y, blockIdx.x, gridDim.x, s_m);
}

// prep_x and x_limbs in one cooperative launch (every block resident): the
// prep work, a grid-wide synchronisation, then the limbs.
__global__ void __launch_bounds__(256) prep_limbs_kernel(Arena A, Work W, const double* __restrict__ x, int n,
                                                         long long ld, int n_chunks, int* zero, int n_zero,
                                                         int* status, int n_pad) {
    __shared__ int s_m[8];
    pdl_trigger();
    prep_block(A, W, x, n, ld, n_chunks, zero, n_zero, status, s_m);
    cooperative_groups::this_grid().sync();
    limbs_block(W, n, n_pad, gridDim.x, blockIdx.y, blockIdx.x, gridDim.x, s_m);
}

// Bring a line into L1 ahead of its use (no register waits on it).
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
// 8-byte asynchronous global -> shared copy (no register held while in flight).
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// A column unit's descriptor from four 16-byte words (shared or global).
__device__ __forceinline__ ColTask load_task(const int4* q) {
    const int4 a = q[0], b = q[1], c = q[2], d = q[3];
    ColTask T;
    T.col0 = a.x, T.n = a.y, T.count = a.z, T.width = a.w;
    T.off = (long long)(((unsigned long long)(unsigned)b.y << 32) | (unsigned)b.x);
    T.stride = b.z, T.comp_idx = b.w;
    T.chunk0 = c.x, T.nchunks = c.y, T.part = c.z, T.nparts = c.w;
    T.split_id = d.x, T.cps = d.y;
    T.dest0 = d.z, T.ndest = d.w;
    return T;
}

// Column-side accumulators of one warp: FP32 MMA sums per M-tile and plane
// (exact below 2^24), their 64-bit folds, and the same for sum_i X_i.
struct ColAcc {
    float D[2][4][4];
    long long acc[2][4];
    int since;
};

// Fold the FP32 sums into the 64-bit per-limb sums: plane m < P-1 holds
// subnormal digits (sums in units of 2^-24), the top plane signed digits
// (units of 1); plane m weighs 2^(8m).
template <int P>
__device__ __forceinline__ void col_fold(ColAcc& a) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            long long v = 0;
#pragma unroll
            for (int m = 0; m < P; ++m) {
                const float d = m == P - 1 ? a.D[q][m][r] : a.D[q][m][r] * 16777216.0f;
                v += (long long)__float2int_rn(d) << (8 * m);
                a.D[q][m][r] = 0.f;
            }
            a.acc[q][r] += v;
        }
    a.since = 0;
}

// The chunks of a step of a task with P planes (nibble top plane if nibtop):
// per chunk, the x limbs' B fragments and two MMAs per (M-tile, plane) group.
template <int P>
__device__ __forceinline__ void col_step(ColAcc& a, const uint8_t* slot, int nc, int stride, int count, bool nibtop,
                                         uint32_t hb, int g, int t, int lane) {
    const int RB = (P - 1) * 32 + (nibtop ? 16 : 32);  // bytes of one row over all planes
    const uint32_t xrow = smem_u32(slot + nc * stride) + 16u * unsigned(lane);
    const int rows0 = count < 16 ? count : 16, rows1 = count - 16;
    for (int c = 0; c < nc; ++c) {
        const uint8_t* cb = slot + c * stride;
        uint32_t b[4];
        limb_frags(xrow + unsigned(c * kColChunk * 16), b);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int rows = q ? rows1 : rows0;
            if (rows <= 0) break;
            const uint8_t* off = cb + q * 16 * RB;
#pragma unroll
            for (int m = 0; m < P - 1; ++m) {
                group_mma(a.D[q][m], off, false, rows, g, t, b);
                off += rows * 32;
            }
            group_mma_top(a.D[q][P - 1], off, nibtop, rows, g, t, b, hb);
        }
        if (++a.since == 8) col_fold<P>(a);
    }
}

// A dense unit of the column side: columns [k0, k0 + nc) of a dense diagonal
// block part of one row tile for rhs column p, lane l owning tile rows l and
// l + 32 (columns in order, FP64; consecutive lanes read consecutive doubles),
// stored as the unit's row-sum slice.  The FP64 pipe is the scarce one on
// this GPU, so the blocks are cut into many short units that spread over all
// schedulers and run beside the other warps' integer and tensor-core work.
__device__ __forceinline__ void dense_unit(const Arena& A, const Work& W, const ColTask& u, int p, int n,
                                           int n_dslices, int lane) {
    const int rows = __ldg(&A.tiles[u.stride].rows);
    const TileDense D = A.tdense[u.col0];
    const bool r0 = lane < rows, r1 = lane + 32 < rows;
    const double* col = A.dense + D.off + (long long)u.chunk0 * D.ld + lane;
    const double* xv = W.xc + (long long)p * n + D.xcol + u.chunk0;
    double s0 = 0.0, s1 = 0.0;
    // batches of eight columns: every load of a batch is issued before its
    // FMAs (the dense data comes from HBM); rows past the tile read 0 and add
    // nothing (fma(0, x, s) = s for finite x)
    int k = 0;
    for (; k + 8 <= u.n; k += 8) {
        double c0[8], c1[8], xk[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            xk[i] = __ldcg(xv + k + i);
            c0[i] = r0 ? __ldg(col + (long long)(k + i) * D.ld) : 0.0;
            c1[i] = r1 ? __ldg(col + (long long)(k + i) * D.ld + 32) : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            s0 = fma(c0[i], xk[i], s0);
            s1 = fma(c1[i], xk[i], s1);
        }
    }
    for (; k < u.n; ++k) {
        const double xk = __ldcg(xv + k);
        if (r0) s0 = fma(__ldg(col + (long long)k * D.ld), xk, s0);
        if (r1) s1 = fma(__ldg(col + (long long)k * D.ld + 32), xk, s1);
    }
    double* out = W.pdense + ((long long)p * n_dslices + u.comp_idx) * 64;
    out[lane] = s0;
    out[lane + 32] = s1;
}

// Column side.  Warp gw owns the units warp_off[gw] .. warp_off[gw + 1]
// (assigned longest first at upload by a per-unit cycle model, heaviest first
// per warp; the first kStagedUnits descriptors are kept in shared memory); its
// work is the sequence (unit, rhs column, chunk), streamed through a
// kColStages-deep pipeline of shared-memory slots filled by bulk copies (the
// chunks' code groups and the limbs of their x entries), kColStages - 1 steps
// ahead of their use.  Per chunk the warp runs, for each M-tile and digit
// plane, two 16x8x16 MMAs (digits x the eight x limbs; the top plane's digits
// signed); the FP32 sums are folded into 64-bit integers every 8 chunks
// (before any can reach 2^24).  At the unit's end the limbs and planes are
// combined into exact 128-bit sums t_j = sum_i c_ij X_i (lane j: component j,
// through shared memory), u_j = (s^P s^Q) t_j 2^(xe - 1022 - kFixBits), and
// the B rows of u_j on each consuming tile's exponent are written.  Dense
// units (width 0) are computed in FP64 by dense_unit.
__global__ void __launch_bounds__(kWarps * 32, QH_COL_CTAS) column_kernel(Arena A, Work W, const int* __restrict__ warp_off,
                                                                int n_pad, int rhs, int n_split, int n_slots,
                                                                int n, int n_dslices, int* status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t s_bar[kWarps][kColStages];
    __shared__ int2 s_td[kWarps][32];  // each lane's first B row record of the current unit
    __shared__ int4 s_desc[kWarps][kStagedUnits * 4];  // the warp's first unit descriptors
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    uint8_t* slots = smem_raw + (size_t)warp * kColStages * kColSlotBytes;
    uint64_t* bar = s_bar[warp];
    if (lane == 0) {
        for (int i = 0; i < kColStages; ++i) mbar_init(bar + i, 1);
        mbar_init_fence();
    }
    __syncwarp();
    const int gw = blockIdx.x * kWarps + warp;
    const int u0 = __ldg(warp_off + gw), my_units = __ldg(warp_off + gw + 1) - u0;
    const ColTask* my_tasks = A.tasks + u0;
    // the warp's first kStagedUnits descriptors into shared memory (read-only
    // layout: before waiting for the preceding kernel)
    {
        const int4* src = reinterpret_cast<const int4*>(my_tasks);
        const int nst = min(my_units, kStagedUnits) * 4;
        for (int i = lane; i < nst; i += 32) s_desc[warp][i] = __ldg(src + i);
        __syncwarp();
    }
    auto unit = [&](int k) {
        if (k < kStagedUnits) return load_task(&s_desc[warp][4 * k]);
        const int4* q = reinterpret_cast<const int4*>(my_tasks + k);
        const int4 gq[4] = {__ldg(q), __ldg(q + 1), __ldg(q + 2), __ldg(q + 3)};
        return load_task(gq);
    };
    if (my_units <= 0) pdl_wait();  // (every thread waits before exiting)
    unsigned issued = 0, computed = 0;  // running step counters (slot, phase)
    ColAcc a;
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int r = 0; r < 4; ++r) a.D[q][m][r] = 0.f;
#pragma unroll
    for (int r = 0; r < 4; ++r) a.acc[0][r] = a.acc[1][r] = 0;
    a.since = 0;
    pdl_trigger();
    if (my_units > 0) {
        const int nb = my_units;
        int ik = 0, ip = 0, ic = 0;  // issue cursor
        ColTask di = unit(0);
        // The first stages' code bytes come from the read-only arena, so they
        // are fetched while the preceding kernel finishes; their x limbs only
        // after it has (programmatic dependent launch): deferred copies.
        bool defer = true;
        int npend = 0;
        const void* pend_src[kColStages];
        uint8_t* pend_dst[kColStages];
        unsigned pend_bytes[kColStages], pend_slot[kColStages];
        auto issue = [&]() {
            while (ik < nb && di.width == 0) {  // dense units stream nothing
                if (++ik < nb) di = unit(ik);
            }
            if (ik >= nb) return;
            const int nc = min(di.cps, di.nchunks - ic);
            const unsigned slot_i = issued % kColStages;
            uint8_t* slot = slots + slot_i * kColSlotBytes;
            const unsigned wbytes = unsigned(nc * di.stride);
            const unsigned xbytes = unsigned(nc * kColChunk * 16);
            const long long k0 = (long long)(di.chunk0 + ic) * kColChunk;
            if (lane == 0) {
                fence_async_smem();
                mbar_arrive_expect(bar + slot_i, wbytes + xbytes);
                bulk_load(slot, A.qcodes + di.off + (long long)(di.chunk0 + ic) * di.stride, wbytes, bar + slot_i);
                const void* xsrc = W.xq + (long long)ip * n_pad + di.col0 + k0;
                if (defer) {
                    pend_src[npend] = xsrc, pend_dst[npend] = slot + wbytes;
                    pend_bytes[npend] = xbytes, pend_slot[npend] = slot_i;
                    ++npend;
                } else {
                    bulk_load(slot + wbytes, xsrc, xbytes, bar + slot_i);
                }
            }
            ++issued;
            ic += nc;
            if (ic == di.nchunks) {
                ic = 0;
                if (++ip == rhs) {
                    ip = 0;
                    if (++ik < nb) {
                        di = unit(ik);
                    }
                }
            }
        };
        __syncwarp();
        int ck = 0, cp = 0, cc = 0;  // compute cursor (first unit: before the issue cursor moves on)
        ColTask dc = di;
#pragma unroll 1
        for (int s = 0; s < kColStages - 1; ++s) issue();
        pdl_wait();  // x limbs and exponents of this apply
        defer = false;
        if (lane == 0)
            for (int i = 0; i < npend; ++i) bulk_load(pend_dst[i], pend_src[i], pend_bytes[i], bar + pend_slot[i]);
        const int xe0 = W.xe[0];
        // this lane's component scale and first B row record, loaded when a
        // unit starts (the record by an asynchronous copy into shared
        // memory) and used at its end
        double rec = 0.0;
        int2* my_td = &s_td[warp][lane];
        auto load_rec = [&]() {
            if (lane < dc.count) rec = __ldg(&A.task_rec[dc.comp_idx + lane].scale);
            if (lane < dc.ndest) cp_async8(my_td, A.task_dest + dc.dest0 + lane);
        };
        load_rec();
        while (ck < nb) {
            if (dc.width == 0) {  // dense unit: no stage
                dense_unit(A, W, dc, cp, n, n_dslices, lane);
                if (++cp == rhs) {
                    cp = 0;
                    if (++ck < nb) {
                        dc = unit(ck);
                        load_rec();
                    }
                }
                continue;
            }
            issue();
            const unsigned slot_i = computed % kColStages;
            if (!mbar_wait(bar + slot_i, (computed / kColStages) & 1)) {
                flag_timeout(status);
                break;
            }
            const int nc = min(dc.cps, dc.nchunks - cc);
            const uint8_t* slot = slots + slot_i * kColSlotBytes;
            const int P = (dc.width + 7) >> 3;
            const int tb = dc.width - 8 * (P - 1);  // bits of the top digit
            const bool nibtop = tb <= 4;
            const uint32_t hb = (0x6400u | (1u << (tb - 1))) * 0x00010001u;
            switch (P) {
                case 1: col_step<1>(a, slot, nc, dc.stride, dc.count, nibtop, hb, g, t, lane); break;
                case 2: col_step<2>(a, slot, nc, dc.stride, dc.count, nibtop, hb, g, t, lane); break;
                case 3: col_step<3>(a, slot, nc, dc.stride, dc.count, nibtop, hb, g, t, lane); break;
                default: col_step<4>(a, slot, nc, dc.stride, dc.count, nibtop, hb, g, t, lane); break;
            }
            ++computed;
            cc += nc;
            if (cc == dc.nchunks) {
                switch ((dc.width + 7) >> 3) {
                    case 1: col_fold<1>(a); break;
                    case 2: col_fold<2>(a); break;
                    case 3: col_fold<3>(a); break;
                    default: col_fold<4>(a); break;
                }
                // this lane's per-limb sums: rows 16q + g + 8h, limbs 2t, 2t+1.
                // Unsplit task: stage all rows' sums in the consumed slot (not
                // refilled before the next issue) and let lane j finish row j;
                // a part of a split task adds its sums exactly with atomics and
                // the part that finishes last finishes the rows.
                const int xe = cp == 0 ? xe0 : W.xe[cp];
                long long* st = reinterpret_cast<long long*>(const_cast<uint8_t*>(slot));
                bool finish = true;
                if (dc.nparts == 1) {
#pragma unroll
                    for (int q = 0; q < 2; ++q)
#pragma unroll
                        for (int hh = 0; hh < 2; ++hh) {
                            const int row = 16 * q + 8 * hh + g;
                            *reinterpret_cast<longlong2*>(st + row * 8 + 2 * t) =
                                make_longlong2(a.acc[q][2 * hh], a.acc[q][2 * hh + 1]);
                        }
                } else {
                    long long* blk = W.lsplit + ((long long)cp * n_split * 33 + dc.split_id * 33) * 8;
#pragma unroll
                    for (int q = 0; q < 2; ++q)
#pragma unroll
                        for (int hh = 0; hh < 2; ++hh) {
                            const int row = 16 * q + 8 * hh + g;
                            if (row >= dc.count) continue;
                            unsigned long long* dst = reinterpret_cast<unsigned long long*>(blk + row * 8 + 2 * t);
                            atomicAdd(dst, (unsigned long long)a.acc[q][2 * hh]);
                            atomicAdd(dst + 1, (unsigned long long)a.acc[q][2 * hh + 1]);
                        }
                    __threadfence();
                    __syncwarp();
                    int done = 0;
                    if (lane == 0) done = atomicAdd(W.split_cnt + (long long)cp * n_split + dc.split_id, 1);
                    done = __shfl_sync(0xFFFFFFFFu, done, 0);
                    finish = done == dc.nparts - 1;
                    if (finish) {
                        __threadfence();
                        if (lane < dc.count) {
                            const longlong2* src = reinterpret_cast<const longlong2*>(blk + lane * 8);
#pragma unroll
                            for (int l = 0; l < 4; ++l)
                                *reinterpret_cast<longlong2*>(st + lane * 8 + 2 * l) = __ldcg(src + l);
                        }
                    }
                }
                if (finish) {
                    for (int l = 32 + 16 * lane; l < dc.ndest; l += 512)  // the rest of a long B row list
                        prefetch_l2(A.task_dest + dc.dest0 + l);
                    __syncwarp();
                    // lane j: u of component row j
                    double u = 0.0;
                    if (lane < dc.count) {
                        const longlong2* r2 = reinterpret_cast<const longlong2*>(st + lane * 8);
                        __int128 S = 0;
#pragma unroll
                        for (int l = 0; l < 4; ++l) {
                            const longlong2 v = r2[l];
                            S += ((__int128)v.x << (16 * l)) + ((__int128)v.y << (16 * l + 8));
                        }
                        u = xe ? i128_ldexp(S, xe - 1022 - kFixBits) * rec : 0.0;
                    }
                    // the task's B rows, lanes over the (component, slot)
                    // pairs: U on the tile's exponent and its limbs
                    const int2* tdp = reinterpret_cast<const int2*>(A.task_dest + dc.dest0);
                    cp_async_wait_all();  // this lane's first record
                    for (int d0 = 0; d0 < dc.ndest; d0 += 128) {
                        int2 td[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int d = d0 + 32 * j + lane;
                            td[j] = d < dc.ndest ? (d0 + j == 0 ? *my_td : __ldg(tdp + d)) : make_int2(-1, 0);
                        }
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            if (d0 + 32 * j >= dc.ndest) break;
                            const double ud = __shfl_sync(0xFFFFFFFFu, u, (td[j].y >> 16) & 31);
                            if (td[j].x >= 0) {
                                const int ce = int(int16_t(td[j].y & 0xFFFF));
                                const long long U = to_fixed(ud, xe + ce);  // (0 for 0)
                                W.blimb[(long long)cp * n_slots + td[j].x] = to_limbs(U);
                            }
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < 2; ++q)
#pragma unroll
                    for (int r = 0; r < 4; ++r) a.acc[q][r] = 0;
                cc = 0;
                if (++cp == rhs) {
                    cp = 0;
                    if (++ck < nb) {
                        dc = unit(ck);
                        load_rec();
                    }
                }
            }
            __syncwarp();
        }
    }
    // copies still in flight (only after a failed wait): wait for them, bounded
    while (computed < issued) {
        mbar_wait(bar + computed % kColStages, (computed / kColStages) & 1);
        ++computed;
    }
}

// A row k-pair's info byte: planes | nibble top plane << 3 | (top bits - 1) << 4.
// Bytes of its digit groups, and the top plane's conversion constant.
__device__ __forceinline__ int kp_bytes(int info) { return (info & 7) * 512 - ((info >> 3) & 1) * 256; }
__device__ __forceinline__ uint32_t kp_hb(int info) { return (0x0400u | (1u << (info >> 4))) * 0x00010001u; }

// A row unit's descriptor (four 16-byte loads, cached in L1).
struct RowDesc {
    long long code_off, kp_off;
    int tile, q, h, H, nkps, K, slot0, nsteps, step0;
};

__device__ __forceinline__ RowDesc load_rdesc(const RowUnit* p) {
    const int4* q = reinterpret_cast<const int4*>(p);
    const int4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), e = __ldg(q + 3);
    RowDesc d;
    d.tile = a.x, d.q = a.y, d.h = a.z, d.H = a.w;
    d.nkps = b.x, d.K = b.y, d.slot0 = b.z, d.nsteps = b.w;
    d.code_off = (long long)(((unsigned long long)(unsigned)c.y << 32) | (unsigned)c.x);
    d.kp_off = (long long)(((unsigned long long)(unsigned)c.w << 32) | (unsigned)c.z);
    d.step0 = e.x;
    return d;
}

// The digit groups of one k-pair with P planes (nibble top plane if NIBTOP),
// at compile-time offsets.
template <int P, bool NIBTOP>
__device__ __forceinline__ void kp_groups(float (&D)[4][4], const uint8_t* gp, int g, int t, const uint32_t (&b)[4],
                                          uint32_t hb) {
#pragma unroll
    for (int m = 0; m < P - 1; ++m) {
        group_mma(D[m], gp, false, 16, g, t, b);
        gp += 512;
    }
    group_mma_rtop(D[P - 1], gp, NIBTOP, g, t, b, hb);
}

// Row side.  Warp gw owns the units warp_off[gw] .. warp_off[gw + 1]
// (assigned longest first at upload).  A
// low-rank unit (rows 16q.. of a tile, k-pairs h, h + H, ...) streams its
// digit groups and B rows through a kRowStages-deep bulk-copy pipeline; per
// k-pair it runs, for each plane, two 16x8x16 MMAs of its 16 rows of digits by
// the components' U limbs, folding the FP32 sums into 64-bit integers every 8
// k-pairs (at most 16 k-blocks, below 2^24).  At the end the limbs and planes
// of each row are combined into an exact 128-bit sum and stored as the unit's
// partial.  combine_kernel adds the partials and the dense diagonal blocks.
__global__ void __launch_bounds__(kWarps * 32, QH_ROW_CTAS) row_kernel(Arena A, Work W, const int* __restrict__ warp_off,
                                                             int rhs, int n_slots, int n_tiles, int* status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t s_bar[kWarps][kRowStages];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    uint8_t* slots = smem_raw + (size_t)warp * kRowStages * kRowSlotBytes;
    uint64_t* bar = s_bar[warp];
    if (lane == 0) {
        for (int i = 0; i < kRowStages; ++i) mbar_init(bar + i, 1);
        mbar_init_fence();
    }
    __syncwarp();
    const int gw = blockIdx.x * kWarps + warp;
    const int u0 = __ldg(warp_off + gw), my_units = __ldg(warp_off + gw + 1) - u0;
    const RowUnit* my_units_p = A.units + u0;
    unsigned issued = 0, computed = 0;
    pdl_trigger();
    if (my_units <= 0) pdl_wait();
    if (my_units > 0) {
        const int nb = my_units;
        // issue cursor: unit ik, rhs column ip, step is (k-pair index ii,
        // byte offset ioff); the unit's step words isb .. isb + 31, one per lane
        int ik = 0, ip = 0, is = 0, isb = 0, ii = 0;
        long long ioff = 0;
        RowDesc di = load_rdesc(my_units_p);
        if (lane < 2 && lane + 1 < nb) prefetch_l1(my_units_p + lane + 1);
        // The first stages' code bytes come from the read-only arena, so they
        // are fetched while the column kernel finishes; their B rows only
        // after it has (programmatic dependent launch): deferred copies.
        bool defer = true;
        int npend = 0;
        const void* pend_src[kRowStages];
        uint8_t* pend_dst[kRowStages];
        unsigned pend_bytes[kRowStages], pend_slot[kRowStages];
        auto load_steps = [&](const RowDesc& d, int base) {
            return base + lane < d.nsteps ? __ldg(A.row_steps + d.step0 + base + lane) : 0u;
        };
        auto load_info = [&](const RowDesc& d, int base) {
            return base + lane < d.nkps ? int(__ldg(A.kp_info + d.kp_off + d.h + (base + lane) * d.H)) : 0;
        };
        uint32_t isteps = load_steps(di, 0);
        auto issue = [&]() {
            if (ik >= nb) return;
            if (is - isb == 32) {
                isb = is;
                isteps = load_steps(di, isb);
            }
            const uint32_t sw = __shfl_sync(0xFFFFFFFFu, isteps, is - isb);
            const int c = int(sw & 255u);
            const int cbytes = int((sw >> 8) & 255u) * 256;
            const unsigned slot_i = issued % kRowStages;
            uint8_t* slot = slots + slot_i * kRowSlotBytes;
            const unsigned lbytes = unsigned(c * 512);
            if (lane == 0) {
                fence_async_smem();
                mbar_arrive_expect(bar + slot_i, unsigned(cbytes) + lbytes);
                bulk_load(slot, A.pcodes + di.code_off + ioff, unsigned(cbytes), bar + slot_i);
                const void* bsrc = W.blimb + (long long)ip * n_slots + di.slot0 + 32 * ii;
                if (defer) {
                    pend_src[npend] = bsrc, pend_dst[npend] = slot + cbytes;
                    pend_bytes[npend] = lbytes, pend_slot[npend] = slot_i;
                    ++npend;
                } else {
                    bulk_load(slot + cbytes, bsrc, lbytes, bar + slot_i);
                }
            }
            ++issued;
            ++is;
            ii += c;
            ioff += cbytes;
            if (is == di.nsteps) {
                is = isb = ii = 0;
                ioff = 0;
                if (++ip == rhs) {
                    ip = 0;
                    if (++ik < nb) {
                        di = load_rdesc(my_units_p + ik);
                        if (ik + 2 < nb && lane == 0) prefetch_l1(my_units_p + ik + 2);
                        // the next unit's step words and k-pair infos
                        if (ik + 1 < nb && lane == 0) {
                            const RowDesc dn = load_rdesc(my_units_p + ik + 1);
                            prefetch_l1(A.row_steps + dn.step0);
                            prefetch_l1(A.kp_info + dn.kp_off + dn.h);
                        }
                    }
                }
                isteps = load_steps(di, 0);
            }
        };
        __syncwarp();
        // compute cursor: unit ck, rhs column cp, step cs (words csb ..), k-pair
        // index ci (infos cib ..); first unit: before the issue cursor moves on
        int ck = 0, cp = 0, cs = 0, csb = 0, ci = 0, cib = 0;
        RowDesc dc = di;
#pragma unroll 1
        for (int s = 0; s < kRowStages - 1; ++s) issue();
        pdl_wait();  // B rows of this apply
        defer = false;
        if (lane == 0)
            for (int i = 0; i < npend; ++i) bulk_load(pend_dst[i], pend_src[i], pend_bytes[i], bar + pend_slot[i]);
        uint32_t csteps = load_steps(dc, 0);
        int cinfo = load_info(dc, 0);
        float D[4][4];
        long long acc[4];
        int since = 0;
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int r = 0; r < 4; ++r) D[m][r] = 0.f;
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[r] = 0;
        auto fold_row = [&]() {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                long long v = 0;
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    v += fold(D[m][r], m);
                    D[m][r] = 0.f;
                }
                acc[r] += v;
            }
            since = 0;
        };
        auto advance = [&]() {
            if (++cp == rhs) {
                cp = 0;
                if (++ck < nb) dc = load_rdesc(my_units_p + ck);
            }
            cs = csb = ci = cib = 0;
            csteps = load_steps(dc, 0);
            cinfo = load_info(dc, 0);
        };
        while (ck < nb) {
            issue();
            const unsigned slot_i = computed % kRowStages;
            if (!mbar_wait(bar + slot_i, (computed / kRowStages) & 1)) {
                flag_timeout(status);
                break;
            }
            const uint8_t* slot = slots + slot_i * kRowSlotBytes;
            if (cs - csb == 32) {
                csb = cs;
                csteps = load_steps(dc, csb);
            }
            const uint32_t sw = __shfl_sync(0xFFFFFFFFu, csteps, cs - csb);
            const int c = int(sw & 255u);
            const int cbytes = int((sw >> 8) & 255u) * 256;
            const uint8_t* gp = slot;
            const uint32_t lrow = smem_u32(slot + cbytes) + 16u * unsigned(lane);
            // a uniform step: one digit pattern, no k slot past the k axis
            auto run = [&](auto P_, auto NIB_) {
                constexpr int P = decltype(P_)::value;
                constexpr bool NIB = decltype(NIB_)::value;
                const uint32_t hb = kp_hb(int((sw >> 16) & 255u));
                for (int k = 0; k < c; ++k) {
                    uint32_t b[4];
                    limb_frags(lrow + unsigned(k * 512), b);
                    kp_groups<P, NIB>(D, gp, g, t, b, hb);
                    gp += P * 512 - (NIB ? 256 : 0);
                    if (++since == 8) fold_row();
                }
            };
            using I1 = std::integral_constant<int, 1>;
            using I2 = std::integral_constant<int, 2>;
            using I3 = std::integral_constant<int, 3>;
            using I4 = std::integral_constant<int, 4>;
            if (sw >> 24) {
                switch ((sw >> 16) & 15u) {
                    case 4: run(I4{}, std::false_type{}); break;
                    case 4 | 8: run(I4{}, std::true_type{}); break;
                    case 3: run(I3{}, std::false_type{}); break;
                    case 3 | 8: run(I3{}, std::true_type{}); break;
                    case 2: run(I2{}, std::false_type{}); break;
                    case 2 | 8: run(I2{}, std::true_type{}); break;
                    case 1: run(I1{}, std::false_type{}); break;
                    default: run(I1{}, std::true_type{}); break;
                }
            } else
            for (int k = 0; k < c; ++k) {
                if (ci + k - cib >= 32) {
                    cib = ci + k;
                    cinfo = load_info(dc, cib);
                }
                const int kp = dc.h + (ci + k) * dc.H;
                const int info = __shfl_sync(0xFFFFFFFFu, cinfo, ci + k - cib);
                uint32_t b[4];
                limb_frags(lrow + unsigned(k * 512), b);
                const int kv = dc.K - 32 * kp;  // k slots of this k-pair inside the k axis
                if (kv < 32) {
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int e = 8 * i + 2 * t;
                        if (e >= kv) b[i] &= 0xFFFF0000u;
                        if (e + 1 >= kv) b[i] &= 0x0000FFFFu;
                    }
                }
                const uint32_t hb = kp_hb(info);
                switch (info & 15) {  // planes | nibble top << 3
                    case 4: kp_groups<4, false>(D, gp, g, t, b, hb); break;
                    case 4 | 8: kp_groups<4, true>(D, gp, g, t, b, hb); break;
                    case 3: kp_groups<3, false>(D, gp, g, t, b, hb); break;
                    case 3 | 8: kp_groups<3, true>(D, gp, g, t, b, hb); break;
                    case 2: kp_groups<2, false>(D, gp, g, t, b, hb); break;
                    case 2 | 8: kp_groups<2, true>(D, gp, g, t, b, hb); break;
                    case 1: kp_groups<1, false>(D, gp, g, t, b, hb); break;
                    default: kp_groups<1, true>(D, gp, g, t, b, hb); break;
                }
                gp += kp_bytes(info);
                if (++since == 8) fold_row();
            }
            ++computed;
            ci += c;
            if (++cs == dc.nsteps) {
                fold_row();
                // row g + 8(t&1): limbs over the row's four lanes
                __int128 v0 = ((__int128)acc[0] << (16 * t)) + ((__int128)acc[1] << (16 * t + 8));
                __int128 v1 = ((__int128)acc[2] << (16 * t)) + ((__int128)acc[3] << (16 * t + 8));
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[r] = 0;
                const bool hi = t & 1;
                __int128 R = hi ? v1 : v0;
                R += shfl_xor_i128(hi ? v0 : v1, 1);
                R += shfl_xor_i128(R, 2);
                const long long tb = ((long long)cp * n_tiles + dc.tile) * kTileUnits;
                if (t < 2) st_i128(W.plr + (tb + dc.q * dc.H + dc.h) * 16 + g + 8 * t, R);
                advance();
            }
            __syncwarp();
        }
    }
    // copies still in flight (only after a failed wait): wait for them, bounded
    while (computed < issued) {
        mbar_wait(bar + computed % kRowStages, (computed / kRowStages) & 1);
        ++computed;
    }
}

// One CTA of 64 threads per (row tile, rhs column), one thread per row: y =
// the tile's dense slices (column side) added in column order + the low-rank
// row sums of the tile's units, converted once.
__global__ void __launch_bounds__(64) combine_kernel(Arena A, Work W, double* __restrict__ y, int n_tiles,
                                                    int n_dslices, long long ld) {
    pdl_trigger();
    const int p = blockIdx.y, tile = blockIdx.x, r = threadIdx.x;
    const RowTile T = A.tiles[tile];
    if (r >= T.rows) {
        pdl_wait();
        return;
    }
    const int out = __ldg(A.perm + T.row0 + r);
    pdl_wait();
    const int xe = W.xe[p];
    const long long tb = ((long long)p * n_tiles + tile) * kTileUnits;
    __int128 R = 0;
    for (int h = 0; h < T.nh; ++h) R += ld_i128(W.plr + (tb + (r >> 4) * T.hsplit + h) * 16 + (r & 15));
    double d = 0.0;
    for (int i = 0; i < T.nds; ++i) d += __ldcg(W.pdense + ((long long)p * n_dslices + T.ds0 + i) * 64 + r);
    const double lr = (xe && T.c_exp != kNoExp) ? i128_ldexp(R, xe + T.c_exp - 1022 - kFixBits) : 0.0;
    y[(long long)out * ld + p] = d + lr;
}

// Validation: decode every code from the resident layout through the same
// fragment routines the apply kernels feed to the MMA (group_digits uses the
// permutes and masks of group_mma).  out[comp_base[c] + i] = code i of
// component c (i: block column on the right side, clustered row on the left).
__global__ void decode_col_kernel(Arena A, int n_tasks, const long long* __restrict__ comp_base, int* out) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int ti = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ti < n_tasks; ti += warps) {
        const ColTask T = A.tasks[ti];
        if (T.width == 0) continue;  // dense unit
        const int P = (T.width + 7) / 8;
        const bool nibtop = T.width - 8 * (P - 1) <= 4;
        const int RB = (P - 1) * 32 + (nibtop ? 16 : 32);
        for (int ch = T.chunk0; ch < T.chunk0 + T.nchunks; ++ch) {
            const uint8_t* cb = A.qcodes + T.off + (long long)ch * T.stride;
            for (int q = 0; q < 2; ++q) {
                const int rows = min(16, T.count - 16 * q);
                if (rows <= 0) continue;
                uint32_t u[2][8] = {};
                int off = q * 16 * RB;
                for (int m = 0; m < P; ++m) {
                    const bool nib = nibtop && m == P - 1;
                    uint32_t d[2][8];
                    group_digits(cb + off, nib, rows, g, t, d);
                    for (int hh = 0; hh < 2; ++hh)
                        for (int k = 0; k < 8; ++k) u[hh][k] |= d[hh][k] << (8 * m);
                    off += rows * (nib ? 16 : 32);
                }
                for (int hh = 0; hh < 2; ++hh) {
                    const int j = 16 * q + 8 * hh + g;
                    if (j >= T.count) continue;
                    const int c = A.task_rec[T.comp_idx + j].comp;
                    for (int k = 0; k < 8; ++k) {
                        const int i = ch * kColChunk + slot_entry(k >> 2, k & 3, t);
                        if (i < T.n) out[comp_base[c] + i] = int(int64_t(u[hh][k]) - (int64_t(1) << (T.width - 1)));
                    }
                }
            }
        }
    }
}

__global__ void decode_row_kernel(Arena A, int n_units, const long long* __restrict__ comp_base, int* out) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int ui = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); ui < n_units; ui += warps) {
        const RowUnit U = A.units[ui];
        const RowTile T = A.tiles[U.tile];
        const uint8_t* gp = A.pcodes + U.code_off;
        for (int i = 0; i < U.nkps; ++i) {
            const int kp = U.h + i * U.H;
            const int info = A.kp_info[U.kp_off + kp];
            const int planes = info & 7, half = 1 << (info >> 4);
            long long u[2][8] = {};
            for (int m = 0; m < planes; ++m) {
                const bool nib = m == planes - 1 && ((info >> 3) & 1);
                uint32_t d[2][8];
                group_digits(gp, nib, 16, g, t, d);
                for (int hh = 0; hh < 2; ++hh)
                    for (int k = 0; k < 8; ++k)
                        u[hh][k] += (m == planes - 1 ? (long long)d[hh][k] - half : (long long)d[hh][k]) << (8 * m);
                gp += nib ? 256 : 512;
            }
            for (int hh = 0; hh < 2; ++hh) {
                const int tr = 16 * U.q + 8 * hh + g;
                if (tr >= T.rows) continue;
                for (int k = 0; k < 8; ++k) {
                    const int e = slot_entry(k >> 2, k & 3, t);
                    const int c = A.slot_rec[U.slot0 + 32 * i + e].comp;
                    if (c < 0) continue;
                    out[comp_base[c] + T.row0 + tr] = int(u[hh][k]);
                }
            }
        }
    }
}

// Dense reconstruction (src/qhmat/core.cpp:392-410): thread per entry of one
// block (blocks by binary search over the entry prefix), value = the dense
// entry or 0, plus, per component in order, (c^P s^P)(c^Q s^Q) with separate
// IEEE multiplies and adds in the reference's order, written to
// out[perm[row] * n + perm[col]].  Codes come from decode_*_kernel
// (component-major: comp_base_l[c] + block row, comp_base_r[c] + block column).
__global__ void reconstruct_kernel(Arena A, int n_lr, int n_dense, const long long* __restrict__ ent0,
                                   long long total, const int* __restrict__ lcodes, const int* __restrict__ rcodes,
                                   const long long* __restrict__ lbase, const long long* __restrict__ rbase,
                                   int n, double* __restrict__ out) {
    const int nb = n_lr + n_dense;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = nb - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ent0[mid] <= e) lo = mid;
            else hi = mid - 1;
        }
        const long long le = e - ent0[lo];
        double value = 0.0;
        int row, col;
        if (lo < n_lr) {
            const LowRankDesc d = A.lr[lo];
            const int i = int(le / d.n), k = int(le % d.n);
            for (int j = 0; j < d.rank; ++j) {
                const int c = d.comp0 + j;
                const double l = __dmul_rn(double(lcodes[lbase[c] + i]), A.comp_sl[c]);
                const double r = __dmul_rn(double(rcodes[rbase[c] + k]), A.comp_sr[c]);
                value = __dadd_rn(value, __dmul_rn(l, r));
            }
            row = d.row0 + i;
            col = d.col0 + k;
        } else {
            const DenseDesc d = A.dd[lo - n_lr];
            const int i = int(le / d.n), k = int(le % d.n);
            value = A.dense[d.off + (long long)k * d.m + i];
            row = d.row0 + i;
            col = d.col0 + k;
        }
        out[(long long)A.perm[row] * n + A.perm[col]] = value;
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

// Shared with the other translation units of the library (errors.hpp).
int set_error(int code, const std::string& msg) { return fail(code, msg); }

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
    // unit schedules: warp w of the column (row) grid runs units
    // warp_off[w] .. warp_off[w + 1] of the (reordered) task (unit) array
    int* sched = nullptr;
    int col_grid = 0, row_grid = 0;
    // lazily allocated scratch for calls without a workspace, and host staging
    std::mutex mu;
    void* own_ws = nullptr;  // qh_matmul_host's device buffer
    size_t own_ws_bytes = 0;
    void* dev_ws = nullptr;  // the workspace of qh_matmul_device calls without one
    size_t dev_ws_bytes = 0;
    double* pinned = nullptr;
    size_t pinned_bytes = 0;
    int* d_status = nullptr;
    int* h_status = nullptr;
    cudaStream_t stream = nullptr;
    // the device reads and writes pageable host memory through the host's
    // page tables (coherent host link): host-buffer applies need no staging
    bool host_direct = false;
    // most blocks of prep_limbs_kernel the device holds at once (0: no
    // cooperative launch)
    int prep_coop_max = 0;
    ~qh_matrix() {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        if (arena) cudaFree(arena);
        if (sched) cudaFree(sched);
        if (own_ws) cudaFree(own_ws);
        if (dev_ws) cudaFree(dev_ws);
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

// Longest-first assignment of n units (cost(i)) to W warps: each unit goes to
// the warp with the least work so far.  Returns the permutation (warp-major,
// each warp's units heaviest first) and the W + 1 warp offsets.
template <class F>
void schedule(int n, int W, F cost, std::vector<int32_t>& order, std::vector<int32_t>& off) {
    std::vector<int32_t> idx(static_cast<size_t>(n), 0);
    std::iota(idx.begin(), idx.end(), 0);
    std::vector<double> c(static_cast<size_t>(n), 0.0);
    for (int i = 0; i < n; ++i) c[size_t(i)] = cost(i);
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return c[size_t(a)] > c[size_t(b)]; });
    using Load = std::pair<double, int32_t>;
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int32_t w = 0; w < W; ++w) heap.push({0.0, w});
    std::vector<std::vector<int32_t>> lists(static_cast<size_t>(W));
    for (int32_t i : idx) {
        Load l = heap.top();
        heap.pop();
        lists[size_t(l.second)].push_back(i);
        l.first += c[size_t(i)];
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

template <class T>
void permute(T* a, const std::vector<int32_t>& order) {
    std::vector<T> tmp(a, a + order.size());
    for (size_t i = 0; i < order.size(); ++i) a[i] = tmp[size_t(order[i])];
}

int upload(Layout&& L, int device, qh_matrix** out) {
    int rc = check_device(device);
    if (rc) return rc;
    DeviceGuard g(device);
    qh_matrix* m = new (std::nothrow) qh_matrix();
    if (!m) return fail(QH_ERUNTIME, "out of host memory");
    m->L = std::move(L);
    m->device = device;
    cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
    {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        m->host_direct = pageable == 1 && host_tables == 1;
        int coop = 0, per_sm = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
        if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prep_limbs_kernel, 256, 0) == cudaSuccess)
            m->prep_coop_max = per_sm * m->sms;
        cudaGetLastError();
    }
    {
        // warp schedules for this device's grids: units longest first, each
        // to the warp with the least predicted time.
        Layout& Lm = m->L;
        m->col_grid = std::max(1, std::min((Lm.n_tasks + kWarps - 1) / kWarps, m->sms * 2));
        m->row_grid = std::max(1, std::min((Lm.n_units + kWarps - 1) / kWarps, m->sms * 2));
        auto* tasks = reinterpret_cast<ColTask*>(Lm.arena.data() + Lm.sec.tasks);
        auto* units = reinterpret_cast<RowUnit*>(Lm.arena.data() + Lm.sec.units);
        const uint8_t* kpi = Lm.arena.data() + Lm.sec.kp_info;
        std::vector<int32_t> corder, coff, rorder, roff;
        schedule(Lm.n_tasks, m->col_grid * kWarps, [&](int i) {
            // SM cycles of a column unit with all warps resident (least
            // squares over clock64 timings of every unit of a 32768-point
            // kernel matrix, R^2 0.97): per unit (descriptor loads, the
            // finalize), per pipeline step (copy latency not hidden by two
            // stages), per chunk and per code byte; per 32 B rows written
            // (timed alone), charged to every part of a split task since any
            // of them may be the one that finishes it
            const ColTask& T = tasks[i];
            if (T.width == 0) return 1000.0 * double(T.n);  // dense unit: FP64, ~16k cycles for 16 columns
            const double steps = double((T.nchunks + T.cps - 1) / T.cps);
            return 4100.0 + 1415.0 * steps + 490.0 * T.nchunks + 0.194 * double(T.nchunks) * T.stride +
                   700.0 * double((T.ndest + 31) / 32) + (T.nparts > 1 ? 584.0 : 0.0);
        }, corder, coff);
        schedule(Lm.n_units, m->row_grid * kWarps, [&](int i) {
            // SM cycles of a row unit with all warps resident (clock64
            // timings of every unit of a 32768-point kernel matrix): per
            // k-pair and per digit plane of it (MMAs, digit conversion), per
            // pipeline step, per unit (descriptor, the 128-bit epilogue)
            const RowUnit& U = units[i];
            double planes = 0;
            for (int k = 0; k < U.nkps; ++k) planes += kpi[U.kp_off + U.h + int64_t(k) * U.H] & 7;
            return 2000.0 + 350.0 * U.nkps + 380.0 * planes + 300.0 * U.nsteps;
        }, rorder, roff);
        permute(tasks, corder);
        permute(units, rorder);
        std::vector<int32_t> sched(coff);
        sched.insert(sched.end(), roff.begin(), roff.end());
        cudaError_t e2 = cudaMalloc(&m->sched, 4 * sched.size());
        if (e2 == cudaSuccess) e2 = cudaMemcpy(m->sched, sched.data(), 4 * sched.size(), cudaMemcpyHostToDevice);
        if (e2 != cudaSuccess) {
            delete m;
            return cuda_fail(e2, "cudaMalloc");
        }
    }
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
    e = cudaFuncSetAttribute(row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kRowPipeSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(column_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kColPipeSmem);
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "cudaFuncSetAttribute");
    }
    // The host image is no longer needed once uploaded.
    std::vector<uint8_t>().swap(m->L.arena);
    const Sections& S = m->L.sec;
    auto* base = static_cast<const uint8_t*>(m->arena);
    m->A.perm = reinterpret_cast<const int32_t*>(base + S.perm);
    m->A.iperm = reinterpret_cast<const int32_t*>(base + S.iperm);
    m->A.lr = reinterpret_cast<const LowRankDesc*>(base + S.lr);
    m->A.dd = reinterpret_cast<const DenseDesc*>(base + S.dd);
    m->A.comp_w = base + S.comp_w;
    m->A.comp_s = reinterpret_cast<const double*>(base + S.comp_s);
    m->A.tasks = reinterpret_cast<const ColTask*>(base + S.tasks);
    m->A.task_rec = reinterpret_cast<const TaskRec*>(base + S.task_rec);
    m->A.qcodes = base + S.qcodes;
    m->A.pcodes = base + S.pcodes;
    m->A.dense = reinterpret_cast<const double*>(base + S.dense);
    m->A.tiles = reinterpret_cast<const RowTile*>(base + S.tiles);
    m->A.units = reinterpret_cast<const RowUnit*>(base + S.units);
    m->A.tdense = reinterpret_cast<const TileDense*>(base + S.tdense);
    m->A.kp_info = base + S.kp_info;
    m->A.slot_rec = reinterpret_cast<const SlotRec*>(base + S.slot_rec);
    m->A.task_dest = reinterpret_cast<const TaskDest*>(base + S.task_dest);
    m->A.row_steps = reinterpret_cast<const uint32_t*>(base + S.row_steps);
    m->A.comp_sl = reinterpret_cast<const double*>(base + S.comp_sl);
    m->A.comp_sr = reinterpret_cast<const double*>(base + S.comp_sr);
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

// Right-hand-side columns one chain of launches handles at most (gridDim.y
// of the prep and combine launches); wider applies run column chunks in
// turn (every column is computed independently, so the result is the same).
constexpr size_t kMaxRhsChunk = 65535;

size_t rhs_chunk(size_t rhs) { return std::min(rhs, kMaxRhsChunk); }

struct WsPlan {
    size_t xc, xblk, xe, xq, lsplit, cnt, blimb, plr, pdense, total, zero0, zero_bytes;
    int nblk;
};

// x limbs are read by whole 32-entry chunks: pad past the last chunk.
size_t padded_order(const Layout& L) { return (L.order + kColChunk - 1) / kColChunk * kColChunk + kColChunk; }

WsPlan ws_plan(const Layout& L, size_t rhs) {
    WsPlan w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += align256(std::max<size_t>(bytes, 1));
        return o;
    };
    w.nblk = (L.n_chunks + 7) / 8;
    // zeroed by prep_x (contiguous): split partial sums and counters
    w.zero0 = off;
    w.lsplit = take(8 * 8 * 33 * size_t(L.n_split) * rhs);
    w.cnt = take(4 * size_t(L.n_split) * rhs);
    w.zero_bytes = off - w.zero0;
    w.xe = take(4 * rhs);
    w.xblk = take(4 * size_t(w.nblk) * rhs);
    w.xc = take(8 * L.order * rhs);
    w.xq = take(16 * padded_order(L) * rhs);
    w.blimb = take(16 * size_t(L.n_slots) * rhs);
    w.plr = take(16 * 16 * kTileUnits * size_t(L.n_tiles) * rhs);
    w.pdense = take(8 * 64 * size_t(L.n_dslices) * rhs);
    w.total = off;
    return w;
}

// Workspace of an apply with rhs columns (one column chunk's worth).
size_t ws_bytes(const Layout& L, size_t rhs) { return ws_plan(L, rhs_chunk(rhs)).total; }

// Launch with programmatic stream serialization (the kernel may start while
// its predecessor finishes; it waits in-kernel for the predecessor's results).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// One chain of launches for columns [c0, c0 + rhs) of x and y (leading
// dimension ld).
int launch_chunk(const qh_matrix* m, const double* x, double* y, size_t rhs, long long ld, void* ws,
                 cudaStream_t s, int* status, void* const* ev) {
    const Layout& L = m->L;
    const int n = int(L.order);
    auto* w = static_cast<uint8_t*>(ws);
    const WsPlan P = ws_plan(L, rhs);
    Work W;
    W.xc = reinterpret_cast<double*>(w + P.xc);
    W.xblk = reinterpret_cast<int*>(w + P.xblk);
    W.xe = reinterpret_cast<int*>(w + P.xe);
    W.xq = reinterpret_cast<uint4*>(w + P.xq);
    W.lsplit = reinterpret_cast<long long*>(w + P.lsplit);
    W.split_cnt = reinterpret_cast<int*>(w + P.cnt);
    W.blimb = reinterpret_cast<uint4*>(w + P.blimb);
    W.plr = reinterpret_cast<uint4*>(w + P.plr);
    W.pdense = reinterpret_cast<double*>(w + P.pdense);
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[i]), s);
    };
    const int irhs = int(rhs);
    mark(0);
    const int n_pad = int(padded_order(L));
    int* zero = reinterpret_cast<int*>(w + P.zero0);
    const int n_zero = int(P.zero_bytes / 4);
    cudaError_t e;
    if (static_cast<long long>(P.nblk) * irhs <= m->prep_coop_max) {
        // one cooperative launch: prep, a grid-wide synchronisation, limbs
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(unsigned(P.nblk), unsigned(rhs));
        cfg.blockDim = dim3(256);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, prep_limbs_kernel, m->A, W, x, n, ld, L.n_chunks, zero, n_zero, status, n_pad);
    } else {
        prep_x_kernel<<<dim3(unsigned(P.nblk), unsigned(rhs)), 256, 0, s>>>(m->A, W, x, n, ld, L.n_chunks, zero,
                                                                            n_zero, status);
        e = launch_pdl(x_limbs_kernel, dim3(unsigned((n_pad + 255) / 256), unsigned(rhs)), dim3(256), 0, s, W, n,
                       n_pad, P.nblk);
    }
    mark(1);
    if (e == cudaSuccess && L.n_tasks > 0)
        e = launch_pdl(column_kernel, dim3(unsigned(m->col_grid)), dim3(kWarps * 32), size_t(kColPipeSmem), s, m->A,
                       W, static_cast<const int*>(m->sched), n_pad, irhs, L.n_split, L.n_slots, n, L.n_dslices, status);
    mark(2);
    if (e == cudaSuccess && L.n_units > 0)
        e = launch_pdl(row_kernel, dim3(unsigned(m->row_grid)), dim3(kWarps * 32), size_t(kRowPipeSmem), s, m->A, W,
                       static_cast<const int*>(m->sched + m->col_grid * kWarps + 1), irhs, L.n_slots, L.n_tiles,
                       status);
    if (e == cudaSuccess)
        e = launch_pdl(combine_kernel, dim3(unsigned(L.n_tiles), unsigned(rhs)), dim3(64), 0, s, m->A, W, y,
                       L.n_tiles, L.n_dslices, ld);
    if (e != cudaSuccess) return cuda_fail(e, "CUDA kernel launch");
    mark(3);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "CUDA kernel launch");
    return QH_OK;
}

// The apply: column chunks of at most kMaxRhsChunk, one chain each, in stream
// order on the same workspace (sized for one chunk).  Events (profiling) are
// recorded around the first chunk's kernels.
int launch(const qh_matrix* m, const double* x, double* y, size_t rhs, void* ws, cudaStream_t s,
           int* status, void* const* ev = nullptr) {
    for (size_t c0 = 0; c0 < rhs; c0 += kMaxRhsChunk) {
        const int rc = launch_chunk(m, x + c0, y + c0, std::min(kMaxRhsChunk, rhs - c0), (long long)rhs, ws, s,
                                    status, c0 == 0 ? ev : nullptr);
        if (rc) return rc;
    }
    return QH_OK;
}

// The reference's checks (src/qhmat/cuda.cu:108-112): a zero or
// overflowing column count is a shape mismatch; more than INT_MAX * 256
// entries is "CUDA launch grid too large".
int check_rhs(const qh_matrix* m, size_t rhs) {
    if (rhs == 0 || rhs > SIZE_MAX / m->L.order) return fail(QH_EINVAL, "right-hand-side shape mismatch");
    if (m->L.order * rhs > size_t(INT32_MAX) * 256) return fail(QH_EOVERFLOW, "CUDA launch grid too large");
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

int qh_matrix_from_batch(const void* const* images, const size_t* lens, size_t count, int device, qh_matrix** out,
                         uint64_t* offsets) {
    if (!out) return fail(QH_EINVAL, "output handle pointer is null");
    *out = nullptr;
    if (!images || !lens || !count) return fail(QH_EINVAL, "empty batch");
    return guarded([&] {
        std::vector<HostMatrix> ms;
        ms.reserve(count);
        for (size_t k = 0; k < count; ++k) ms.push_back(parse_qhmat(static_cast<const uint8_t*>(images[k]), lens[k]));
        std::vector<uint64_t> off;
        // no padding rows: the plain layout's row tiles already stay inside
        // the row slabs of blocks (so inside one matrix), and every row of
        // the block-diagonal matrix must belong to some block
        HostMatrix S = concat_block_diagonal(ms, 1, off);
        std::vector<HostMatrix>().swap(ms);
        Layout L = build_layout(S);
        const int rc = upload(std::move(L), device, out);
        if (rc == QH_OK && offsets)
            for (size_t k = 0; k < count; ++k) offsets[k] = off[k];
        return rc;
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
    const WsPlan P1 = ws_plan(L, 1);
    out->launches_per_apply = (P1.nblk <= m->prep_coop_max ? 2 : 3) + (L.n_tasks > 0) + (L.n_units > 0);
    out->host_direct = m->host_direct ? 1 : 0;
    out->left_code_bytes = L.left_code_bytes;
    out->right_code_bytes = L.right_code_bytes;
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
    if (mm->dev_ws_bytes < need) {
        if (mm->dev_ws) cudaFree(mm->dev_ws);
        mm->dev_ws = nullptr;
        mm->dev_ws_bytes = 0;
        cudaError_t e = cudaMalloc(&mm->dev_ws, need);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
        mm->dev_ws_bytes = need;
    }
    return launch(m, x, y, rhs, mm->dev_ws, static_cast<cudaStream_t>(stream), status, events4);
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
    // Device address of the array, looked up once per device with that device
    // current (the first call on a device does this set-up; a table entry per
    // device the process sees).
    static std::mutex mu;
    static std::vector<void*> addr;
    void* ptr = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (addr.empty()) {
            int count = 0;
            cudaError_t e = cudaGetDeviceCount(&count);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
            addr.assign(size_t(std::max(count, 0)), nullptr);
        }
        if (m->device < 0 || size_t(m->device) >= addr.size()) return fail(QH_EINVAL, "invalid CUDA device ordinal");
        DeviceGuard g(m->device);
        if (!addr[size_t(m->device)]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
            addr[size_t(m->device)] = p;
        }
        ptr = addr[size_t(m->device)];
    }
    DeviceGuard g(m->device);
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
    const auto* xb = reinterpret_cast<const uint8_t*>(x);
    const auto* yb = reinterpret_cast<const uint8_t*>(y);
    if (m->host_direct && (xb + vec <= yb || yb + vec <= xb)) {
        // the kernels read x and write y in the caller's memory directly
        // (each page of y is written once here first, so that the device
        // never touches an unpopulated page)
        if (mm->own_ws_bytes < need_ws) {
            if (mm->own_ws) cudaFree(mm->own_ws);
            mm->own_ws = nullptr;
            mm->own_ws_bytes = 0;
            e = cudaMalloc(&mm->own_ws, need_ws);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
            mm->own_ws_bytes = need_ws;
        }
        {
            // one write per page makes every page of y present and writable
            static const uintptr_t page = uintptr_t(sysconf(_SC_PAGESIZE) > 0 ? sysconf(_SC_PAGESIZE) : 4096);
            const uintptr_t y0 = reinterpret_cast<uintptr_t>(y), y1 = y0 + vec;
            for (uintptr_t a = y0; a < y1; a = (a & ~(page - 1)) + page) *reinterpret_cast<volatile uint8_t*>(a) = 0;
        }
        // the status word is the pinned host int itself (device-accessible at
        // the same address under unified addressing): no memset and no copy
        // back on the stream
        volatile int* hs = mm->h_status;
        *hs = 0;
        rc = launch(m, x, y, rhs, mm->own_ws, mm->stream, mm->h_status);
        if (rc) return rc;
        if ((e = cudaStreamSynchronize(mm->stream)) != cudaSuccess) return cuda_fail(e, "CUDA kernel execution");
        const int st = *hs;
        if (st & kStatusNonfinite) return fail(QH_EINVAL, "nonfinite right-hand side");
        if (st & kStatusTimeout) return fail(QH_ERUNTIME, "device copy wait timed out");
        return QH_OK;
    }
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

int qh_debug_wait_timeout(int device, int polls) {
    if (polls < 1 || polls > (1 << 20)) return fail(QH_EINVAL, "polls must be in [1, 2^20]");
    int rc = check_device(device);
    if (rc) return rc;
    DeviceGuard g(device);
    int* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    int h = 0;
    e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        wait_timeout_kernel<<<1, 32>>>(polls, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "debug wait");
    if (h & kStatusTimeout) return fail(QH_ERUNTIME, "device copy wait timed out");
    return QH_OK;
}

int qh_matrix_reconstruct(const qh_matrix* m, double* out, size_t out_count, int out_on_device) {
    if (!m) return fail(QH_EINVAL, "null matrix handle");
    const size_t n = m->L.order;
    if (n > SIZE_MAX / n / sizeof(double)) return fail(QH_EOVERFLOW, "dense output size overflow");
    if (!out || out_count != n * n) return fail(QH_EINVAL, "output size does not match order * order");
    return guarded([&] {
        DeviceGuard g(m->device);
        int rc = QH_OK;
        const int n_lr = m->L.n_lr, n_dense = m->L.n_dense, nb = n_lr + n_dense;
        std::vector<LowRankDesc> lr(static_cast<size_t>(n_lr));
        std::vector<DenseDesc> dd(static_cast<size_t>(n_dense));
        cudaError_t e = cudaSuccess;
        if (n_lr) e = cudaMemcpy(lr.data(), m->A.lr, sizeof(LowRankDesc) * lr.size(), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && n_dense)
            e = cudaMemcpy(dd.data(), m->A.dd, sizeof(DenseDesc) * dd.size(), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy device-to-host");
        // code offsets (component-major, as qh_debug_decode lays them out) and
        // the entry prefix of the blocks
        std::vector<long long> lbase(size_t(m->L.n_comp) + 1, 0), rbase(size_t(m->L.n_comp) + 1, 0);
        for (const auto& d : lr)
            for (int j = 0; j < d.rank; ++j) {
                lbase[size_t(d.comp0 + j) + 1] = d.m;
                rbase[size_t(d.comp0 + j) + 1] = d.n;
            }
        for (size_t c = 0; c + 1 < lbase.size(); ++c) {
            lbase[c + 1] += lbase[c];
            rbase[c + 1] += rbase[c];
        }
        const long long ltotal = lbase.back(), rtotal = rbase.back();
        std::vector<long long> lrow(lbase);  // left codes are indexed by clustered row
        for (const auto& d : lr)
            for (int j = 0; j < d.rank; ++j) lrow[size_t(d.comp0 + j)] -= d.row0;
        std::vector<long long> ent0(size_t(nb) + 1, 0);
        for (int b = 0; b < nb; ++b) {
            const long long mm = b < n_lr ? lr[size_t(b)].m : dd[size_t(b - n_lr)].m;
            const long long nn = b < n_lr ? lr[size_t(b)].n : dd[size_t(b - n_lr)].n;
            ent0[size_t(b) + 1] = ent0[size_t(b)] + mm * nn;
        }
        const long long total = ent0[size_t(nb)];
        // device scratch: codes, offsets, entry prefix, and the output if on the host
        std::vector<void*> bufs;
        auto alloc = [&](size_t bytes) -> void* {
            void* p = nullptr;
            if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
            bufs.push_back(p);
            return p;
        };
        auto* d_lc = static_cast<int*>(alloc(4 * size_t(ltotal)));
        auto* d_rc = static_cast<int*>(alloc(4 * size_t(rtotal)));
        auto* d_lb = static_cast<long long*>(alloc(8 * lbase.size()));
        auto* d_lr = static_cast<long long*>(alloc(8 * lbase.size()));
        auto* d_rb = static_cast<long long*>(alloc(8 * rbase.size()));
        auto* d_e0 = static_cast<long long*>(alloc(8 * ent0.size()));
        double* d_out = out_on_device ? out : static_cast<double*>(alloc(8 * n * n));
        if (!d_lc || !d_rc || !d_lb || !d_lr || !d_rb || !d_e0 || !d_out) {
            for (void* p : bufs) cudaFree(p);
            return fail(QH_ERUNTIME, "cudaMalloc: out of device memory");
        }
        e = cudaMemcpy(d_lb, lbase.data(), 8 * lbase.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_lr, lrow.data(), 8 * lrow.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_rb, rbase.data(), 8 * rbase.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(d_e0, ent0.data(), 8 * ent0.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(d_out, 0, 8 * n * n);
        if (e == cudaSuccess) {
            if (m->L.n_tasks)
                decode_col_kernel<<<std::max(1, std::min((m->L.n_tasks + 7) / 8, 4096)), 256>>>(m->A, m->L.n_tasks,
                                                                                              d_rb, d_rc);
            if (m->L.n_units)
                decode_row_kernel<<<std::max(1, std::min((m->L.n_units + 7) / 8, 4096)), 256>>>(m->A, m->L.n_units,
                                                                                              d_lr, d_lc);
            if (total)
                reconstruct_kernel<<<unsigned(std::min<long long>((total + 255) / 256, 65536)), 256>>>(
                    m->A, n_lr, n_dense, d_e0, total, d_lc, d_rc, d_lb, d_rb, int(n), d_out);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e == cudaSuccess && !out_on_device) e = cudaMemcpy(out, d_out, 8 * n * n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(e, "reconstruct");
        for (void* p : bufs) cudaFree(p);
        return rc;
    });
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
        // component-major output: component c's codes start at off[c]; the
        // kernels index left codes by clustered row (base off[c] - row0) and
        // right codes by block column (base off[c])
        std::vector<long long> off(size_t(m->L.n_comp) + 1, 0);
        for (const auto& d : lr)
            for (int j = 0; j < d.rank; ++j)
                off[size_t(d.comp0 + j) + 1] = side == 0 ? d.m : d.n;
        for (size_t c = 0; c + 1 < off.size(); ++c) off[c + 1] += off[c];
        const size_t total = size_t(off.back());
        if (side == 0)
            for (const auto& d : lr)
                for (int j = 0; j < d.rank; ++j) off[size_t(d.comp0 + j)] -= d.row0;
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
                decode_row_kernel<<<std::max(1, std::min((m->L.n_units + 7) / 8, 4096)), 256>>>(m->A, m->L.n_units, d_off, d_out);
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
