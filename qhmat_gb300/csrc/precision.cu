// GB300 (sm_103a) precision form of the quantized H-matrix apply: many
// right-hand sides at once on the 5th-generation tensor cores.
//
// The plain apply (matvec.cu) streams every code once per right-hand side.
// Here each code digit is streamed once per pass of up to 64 right-hand sides
// and multiplied, as an f16 operand, against all of them at once with
// tcgen05.mma (M = 128, K = 16 per instruction, N = 3p: hi/mid/lo f16 limbs
// of every right-hand side), accumulating in FP32 in tensor memory:
//
//   pf_xmax / pf_xlimbs  x (source order) -> one exponent per column; x' = x
//                        2^(1037-E) split into three f16 limbs, stored as the
//                        rows 3r + l of XT (clustered entry order), read by
//                        2-D tensor copies (cp.async.bulk.tensor, 128-byte
//                        swizzle) straight into the B operand layout;
//   pf_column_kernel     T = Q^T X' for 128 components sharing a column range;
//                        u = (s^P s^Q) T in FP64 (the per-component scale),
//                        stored as FP32 per row-side slot;
//   pf_row_kernel        y = P U' per 128-row tile (U' = three f16 limbs of u
//                        on a per-column exponent), plus the dense diagonal
//                        blocks as three f16 limb tiles against X' limbs;
//                        FP64 partial sums per K split;
//   pf_combine_kernel    y = the partials of each tile summed in FP64, in
//                        order (deterministic), scattered through perm.
//
// Both streaming kernels are persistent and warp-specialised: one warp issues
// the bulk and tensor copies into a ring of shared-memory stages, six (column)
// or eight (row) warps
// turn digit bytes (and U) into f16 operand tiles, one thread issues the
// MMAs, four warps drain the accumulators from tensor memory.  Every wait is
// bounded; a wait that gives up sets QH_STATUS_TIMEOUT and the block winds
// down (after a bounded drain of its copies and MMAs) instead of hanging.
//
// Accuracy: every digit x limb product is exact; sums are FP32 (relative
// error ~2^-24 of the partial sums), x and u carry ~33 bits in their limbs.
// This form is checked against the plain FP64 form and the dense product.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <unistd.h>

#include "../../include/qhmat_gb300.h"
#include "errors.hpp"
#include "layout.hpp"
#include "batch.hpp"
#include "pf_layout.hpp"

namespace qhg {
namespace pf {

// Warp roles of both kernels: warp 0 issues the copies, one thread of warp 1
// the MMAs, warps 2 .. 2+C-1 convert, the last four drain tensor memory (lane
// quarters 0..3).  The row kernel converts U as well as digit planes; it runs
// eight converters (two per scheduler) and keeps its y sums in tensor memory,
// which leaves them the registers.  The column kernel runs six.
template <int CONV, int ASTAGES>
struct Roles {
    static constexpr int kConvWarps = CONV;
    static constexpr int kEpiWarp0 = 2 + CONV;
    static constexpr int kThreads = 32 * (kEpiWarp0 + 4);
    static constexpr int kAStages = ASTAGES;  // digit-plane stages (raw and f16)
};
using ColRoles = Roles<6, 4>;
using RowRoles = Roles<8, 5>;
constexpr int kConvWarp0 = 2;
constexpr int kMaxAStages = 5;
constexpr int kBStages = 2;
constexpr int kNMax = 192;        // N of one pass (3 limbs x 64 right-hand sides)
constexpr int kBTileBytes = kNMax * 128;   // B operand stage (N rows of 64 f16)
constexpr int kURawBytes = kPfK * kPfMaxRhs * 4;  // 64 slots of FP32 u
constexpr int kWaitLimit = 1 << 22;
// K chunks one accumulation segment spans (a kernel template parameter, SEG,
// chosen per handle: 2 by default, 1 for matrices whose tolerance asks for
// it).  The tensor cores add each MMA's products into the FP32 accumulator
// with truncation, so the error of an accumulator grows with its number of
// MMAs (measured: relative error proportional to the chain length); segments
// of a few chunks are drained into round-to-nearest FP32 registers by the
// epilogue warps, from two alternating tensor-memory buffers (columns 0 and
// 256).  On the n=32768 x 64 workload: 2 chunks 4.8e-7 relative to the plain
// form, 1 chunk 2.4e-7 at 4% more time per pass.
constexpr int kDefaultSegChunks = 2;
constexpr int kAccStride = 256;
constexpr int kStatusNonfinite = QH_STATUS_NONFINITE;
constexpr int kStatusTimeout = QH_STATUS_TIMEOUT;

// Shared-memory map (offsets from a 1024-byte-aligned base): the f16 A tiles
// (16 KB each), the f16 B tiles (24 KB), the raw digit planes (8 KB) and, in
// the row kernel, the raw FP32 u of a chunk (16 KB).
template <class R>
struct SmemMap {
    static constexpr int kOffAF16 = 0;
    static constexpr int kOffBF16 = kOffAF16 + R::kAStages * kPfTileBytes;
    static constexpr int kOffARaw = kOffBF16 + kBStages * kBTileBytes;
    static constexpr int kOffBRaw = kOffARaw + R::kAStages * kPfPlaneBytes;
};
constexpr int kSmemColumn = SmemMap<ColRoles>::kOffBRaw + 1024;  // + alignment slack
constexpr int kSmemRow = SmemMap<RowRoles>::kOffBRaw + kBStages * kURawBytes + 1024;
static_assert(kSmemColumn <= 220 * 1024 && kSmemRow <= 220 * 1024, "shared memory budget");
static_assert(ColRoles::kAStages <= kMaxAStages && RowRoles::kAStages <= kMaxAStages, "stage count");

struct Arena {
    const int32_t* perm;
    const PfColItem* col_items;
    const PfComp* comps;
    const int32_t* dests;
    const PfRowItem* row_items;
    const PfRowChunk* chunks;
    const int32_t* col_sched;
    const int32_t* row_sched;
    const uint8_t* qraw;
    const uint8_t* praw;
};

struct Work {
    int* ex;       // [64] exponent field of max |x| per right-hand side
    __half* xt;    // [N][n_ent] f16 limbs of x' (row 3r + l)
    float* ut;     // [n_slots][pu] u per row-side slot
    double* part;  // [n_parts][128][pu] FP64 partial sums of the row side
};

// ------------------------------------------------------------ primitives

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait; gives up when the block has been told to abort, or after
// kWaitLimit tests (then it raises the abort flag and the timeout bit).
__device__ __forceinline__ bool wait_bar(uint64_t* bar, unsigned parity, volatile int* abort_flag, int* status) {
    for (int i = 0; i < kWaitLimit; ++i) {
        if (mbar_try(bar, parity)) return true;
        if ((i & 255) == 255 && *abort_flag) return false;
    }
    *abort_flag = 1;
    if (status) atomicOr(status, kStatusTimeout);
    return false;
}
// Pull a descriptor two items (chunks) ahead into L1, so that the roles that
// read it find it there instead of waiting for L2 at every item.
__device__ __forceinline__ void prefetch_l1(const void* ptr) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(ptr));
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// 2-D tensor copy of the box at (x, y) of a tensor map into shared memory.
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Tensor memory: allocate / free `cols` columns (one warp), the address
// written to shared memory.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, unsigned cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, unsigned cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzled layout: rows of 128 bytes, 8-row groups 1024 bytes apart (stride
// byte offset), start advanced by 32 bytes per K step of 16 f16.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= uint64_t((addr & 0x3FFFFu) >> 4);
    d |= uint64_t(16 >> 4) << 16;    // leading byte offset (unused for swizzled K-major)
    d |= uint64_t(1024 >> 4) << 32;  // stride byte offset
    d |= uint64_t(1) << 46;          // descriptor version
    d |= uint64_t(2) << 61;          // 128-byte swizzle
    return d;
}
// Instruction descriptor: f16 x f16 -> f32, both K-major, M = 128, N.
__host__ __device__ constexpr uint32_t mma_idesc(int n) {
    return (1u << 4) | (uint32_t(n >> 3) << 17) | (uint32_t(128 >> 4) << 24);
}
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Arrive on `bar` when every MMA this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 16 consecutive FP32 columns of this warp's 32 tensor-memory lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Store 16 FP32 columns of this warp's 32 tensor-memory lanes.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

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

// Byte offset of 16-byte chunk c (elements 8c .. 8c+7) of row r in a 128-row
// x 64-f16 tile, 128-byte swizzle.
__device__ __forceinline__ uint32_t swz_chunk(int r, int c) {
    return uint32_t((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// Eight digit bytes of plane m (top plane signed) -> eight f16 values
// d 2^(E-25) for exponent field E: the f16 with exponent field E and mantissa
// bits d is 2^(E-15) + d 2^(E-25); subtracting 2^(E-15) leaves the digit's
// value exactly (a subnormal when E = 1).  The signed top digit is biased by
// 128 first.
__device__ __forceinline__ uint4 digits_to_f16(uint2 w, uint32_t eb, uint32_t sub, bool top) {
    if (top) {
        w.x ^= 0x80808080u;
        w.y ^= 0x80808080u;
    }
    return make_uint4(hsub2(prmt(w.x, eb, 0x4140u), sub), hsub2(prmt(w.x, eb, 0x4342u), sub),
                      hsub2(prmt(w.y, eb, 0x4140u), sub), hsub2(prmt(w.y, eb, 0x4342u), sub));
}

// Convert one digit plane (rows stored with 64 bytes each) into an f16 A
// tile, digits of plane m weighted 2^(8m + 1 + ebias - 25): the column side
// uses ebias = 0 (plane m at 2^(8m-24)), the row side 24 - 8(P-1) (top plane at
// 2^0).  half 0: 128 stored rows; half 1: stored rows are tile rows 0..63
// (64..127 zero); half 2: stored rows are tile rows 64..127 (0..63 zero).
// NT threads (a compile-time count, so that the loop unrolls and each thread
// keeps several independent loads and conversions in flight).
template <int NT>
__device__ __forceinline__ void convert_plane(const uint8_t* raw, uint8_t* tile, int m, int P, int ebias, int half,
                                              int ctid) {
    const uint32_t E = uint32_t(8 * m + 1 + ebias);
    const uint32_t eb = (E << 2) * 0x01010101u;
    const bool top = m == P - 1;
    const uint32_t sub = ((E << 10) | (top ? 0x80u : 0u)) * 0x00010001u;
    constexpr int kIters = (1024 + NT - 1) / NT;
    uint2 w[kIters];
#pragma unroll
    for (int i = 0; i < kIters; ++i) {
        const int idx = ctid + i * NT, r = idx >> 3, c = idx & 7;
        const int sr = half == 0 ? r : (half == 1 ? (r < 64 ? r : -1) : (r >= 64 ? r - 64 : -1));
        w[i] = (idx < 1024 && sr >= 0) ? *reinterpret_cast<const uint2*>(raw + sr * 64 + c * 8) : make_uint2(0u, 0u);
    }
#pragma unroll
    for (int i = 0; i < kIters; ++i) {
        const int idx = ctid + i * NT, r = idx >> 3, c = idx & 7;
        if (idx >= 1024) break;
        const int sr = half == 0 ? r : (half == 1 ? (r < 64 ? r : -1) : (r >= 64 ? r - 64 : -1));
        const uint4 v = sr >= 0 ? digits_to_f16(w[i], eb, sub, top) : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(tile + swz_chunk(r, c)) = v;
    }
}

// 2^k as a float, k clamped to the normal range [-126, 127].
__device__ __forceinline__ float pow2f_clamped(int k) { return __int_as_float((127 + max(-126, min(127, k))) << 23); }
constexpr int kZeroColumn = -(1 << 20);  // ku of a right-hand side that is all zero

__device__ __forceinline__ uint32_t pack_h2(__half a, __half b) {
    return uint32_t(__half_as_ushort(a)) | (uint32_t(__half_as_ushort(b)) << 16);
}

// U of 64 slots (FP32, row stride pu) -> the f16 B tile: row 3r + l holds limb
// l of u' = u 2^(ku[r] + dk) 256^(P-1) for the 64 slots of a chunk with P
// planes (slots >= nvalid: 0; dk = the layout's u_beta minus the item's).
// Pairs of slots are split with packed conversions.
template <int NT>
__device__ __forceinline__ void convert_u(const float* raw, uint8_t* tile, int p, int pu, int nvalid, int P,
                                          const int* ku, int dk, int ctid) {
    constexpr int kIters = (8 * kPfMaxRhs + NT - 1) / NT;
#pragma unroll
    for (int it = 0; it < kIters; ++it) {
        const int idx = ctid + it * NT;
        if (idx >= p * 8) break;
        const int r = idx % p, kg = idx / p;
        // 2^(ku + dk) 256^(P-1): the column's scale on this item's bound
        const float sc = ku[r] == kZeroColumn ? 0.0f : pow2f_clamped(ku[r] + dk + 8 * (P - 1));
        float v[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int k = 8 * kg + s;
            v[s] = k < nvalid ? raw[k * pu + r] * sc : 0.0f;
        }
        uint32_t h[3][4];
#pragma unroll
        for (int s = 0; s < 8; s += 2) {
            const __half2 a = __floats2half2_rn(v[s], v[s + 1]);
            const float2 af = __half22float2(a);
            const float r0 = v[s] - af.x, r1 = v[s + 1] - af.y;
            const __half2 b = __floats2half2_rn(r0, r1);
            const float2 bf = __half22float2(b);
            const __half2 c = __floats2half2_rn(r0 - bf.x, r1 - bf.y);
            h[0][s >> 1] = *reinterpret_cast<const uint32_t*>(&a);
            h[1][s >> 1] = *reinterpret_cast<const uint32_t*>(&b);
            h[2][s >> 1] = *reinterpret_cast<const uint32_t*>(&c);
        }
#pragma unroll
        for (int l = 0; l < 3; ++l)
            *reinterpret_cast<uint4*>(tile + swz_chunk(3 * r + l, kg)) = make_uint4(h[l][0], h[l][1], h[l][2], h[l][3]);
    }
}

// Shared state of one block.
struct Shared {
    uint64_t a_full[kMaxAStages], a_conv[kMaxAStages], a_empty[kMaxAStages];
    uint64_t b_full[kBStages], b_conv[kBStages], b_empty[kBStages];
    uint64_t acc_full[2], acc_empty[2];
    uint64_t drain;
    uint32_t tmem;
    int abort_flag;
    int ex[kPfMaxRhs];
    int ku[kPfMaxRhs];      // row kernel: U' = u 2^(ku + u_beta - item's u_beta); kZeroColumn for x = 0
    float fxscale[kPfMaxRhs];  // column kernel: 2^(24 + E_r - 1037)
    float flitem[4][kPfMaxRhs];  // row kernel, per drain warp: the current item's 2^-(ku + ...) (low-rank sums)
    float fdscale[kPfMaxRhs];  // row kernel: 2^(E_r - 1037) (dense sums, times 2^dense_exp)
};

__device__ __forceinline__ void init_barriers(Shared& S, int astages, int conv_warps) {
    for (int i = 0; i < astages; ++i) {
        mbar_init(&S.a_full[i], 1);
        mbar_init(&S.a_conv[i], conv_warps);
        mbar_init(&S.a_empty[i], 1);
    }
    for (int i = 0; i < kBStages; ++i) {
        mbar_init(&S.b_full[i], 1);
        mbar_init(&S.b_conv[i], conv_warps);
        mbar_init(&S.b_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
        mbar_init(&S.acc_full[i], 1);
        mbar_init(&S.acc_empty[i], 4);
    }
    mbar_init(&S.drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// ------------------------------------------------------------ prep kernels

// Largest exponent field of each right-hand-side column (and the nonfinite
// flag): block b, thread r reads rows 256b .. 256b+255 of column r.
__global__ void __launch_bounds__(64) pf_xmax_kernel(const double* __restrict__ x, long long ld, int n, int p,
                                                     int* ex, int* status) {
    const int r = threadIdx.x;
    if (r >= p) return;
    int m = 0;
    bool bad = false;
    const int i1 = min(n, (blockIdx.x + 1) * 256);
    for (int i = blockIdx.x * 256; i < i1; ++i) {
        const double v = x[(long long)i * ld + r];
        const int e = int((__double_as_longlong(v) >> 52) & 0x7FF);
        bad |= e == 0x7FF;
        m = max(m, e == 0x7FF ? 0 : e);
    }
    if (bad && status) atomicOr(status, kStatusNonfinite);
    atomicMax(ex + r, m);
}

// XT[3r + l][i] = limb l of x'(perm[i], r) = x 2^(1037 - E_r); rows 3p .. N-1
// and entries n .. n_ent-1 are zero.
__global__ void __launch_bounds__(256) pf_xlimbs_kernel(const double* __restrict__ x, long long ld, int n, int p,
                                                        int n_ent, int N, const int32_t* __restrict__ perm,
                                                        const int* __restrict__ ex, __half* __restrict__ xt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_ent) return;
    const long long src = i < n ? (long long)__ldg(perm + i) : -1;
    for (int r = 0; r < p; ++r) {
        const int E = ex[r];
        double v = src >= 0 && E ? x[src * ld + r] : 0.0;
        if (!isfinite(v)) v = 0.0;
        v = scalbn(v, 1037 - E);
        const __half a = __double2half(v);
        const double r1 = v - double(__half2float(a));
        const __half b = __double2half(r1);
        const double r2 = r1 - double(__half2float(b));
        xt[(long long)(3 * r) * n_ent + i] = a;
        xt[(long long)(3 * r + 1) * n_ent + i] = b;
        xt[(long long)(3 * r + 2) * n_ent + i] = __double2half(r2);
    }
    for (int row = 3 * p; row < N; ++row) xt[(long long)row * n_ent + i] = __ushort_as_half(0);
}

// ------------------------------------------------------------ column kernel

// Persistent: block g runs column items col_sched[g] .. col_sched[g+1].
template <int kSegChunks>
__global__ void __launch_bounds__(ColRoles::kThreads, 1) pf_column_kernel(Arena A, Work W,
                                                                          const __grid_constant__ CUtensorMap xmap,
                                                                          int p, int N, int pu, int* status) {
    constexpr int kConvWarps = ColRoles::kConvWarps, kEpiWarp0 = ColRoles::kEpiWarp0, kAStages = ColRoles::kAStages;
    constexpr int kOffAF16 = SmemMap<ColRoles>::kOffAF16, kOffBF16 = SmemMap<ColRoles>::kOffBF16,
                  kOffARaw = SmemMap<ColRoles>::kOffARaw;
    extern __shared__ uint8_t smem_dyn[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
    __shared__ Shared S;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int it0 = __ldg(A.col_sched + blockIdx.x), it1 = __ldg(A.col_sched + blockIdx.x + 1);
    if (tid == 0) {
        init_barriers(S, kAStages, kConvWarps);
        S.abort_flag = 0;
    }
    if (tid < kPfMaxRhs) {
        const int E = tid < p ? W.ex[tid] : 0;
        S.ex[tid] = E;
        S.fxscale[tid] = E ? ldexpf(1.0f, max(-126, min(127, 24 + E - 1037))) : 0.0f;
    }
    if (warp == 1) tmem_alloc(&S.tmem, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    volatile int* abort_flag = &S.abort_flag;

    if (warp == 0) {
        // ---- producer
        if (lane == 0) {
            unsigned ai = 0, bi = 0;
            bool ok = true;
            for (int it = it0; it < it1 && ok; ++it) {
                const PfColItem I = A.col_items[it];
                if (it + 2 < it1) prefetch_l1(A.col_items + it + 2);
                for (int kc = 0; kc < I.nkc && ok; ++kc) {
                    const int sb = bi % kBStages;
                    if (bi >= kBStages) ok = wait_bar(&S.b_empty[sb], ((bi / kBStages) - 1) & 1, abort_flag, status);
                    if (!ok) break;
                    mbar_expect(&S.b_full[sb], unsigned(N * 128));
                    tma_2d(sm + kOffBF16 + sb * kBTileBytes, &xmap, I.e_base + kc * kPfK, 0, &S.b_full[sb]);
                    ++bi;
                    for (int m = 0; m < I.planes; ++m) {
                        const int sa = ai % kAStages;
                        if (ai >= kAStages) ok = wait_bar(&S.a_empty[sa], ((ai / kAStages) - 1) & 1, abort_flag, status);
                        if (!ok) break;
                        mbar_expect(&S.a_full[sa], kPfPlaneBytes);
                        bulk_g2s(sm + kOffARaw + sa * kPfPlaneBytes,
                                 A.qraw + I.a_off + (long long)(kc * I.planes + m) * kPfPlaneBytes, kPfPlaneBytes,
                                 &S.a_full[sa]);
                        ++ai;
                    }
                }
            }
            // copies still in flight after an abort: wait for them (bounded)
            if (!ok) {
                for (unsigned k = ai > kAStages ? ai - kAStages : 0; k < ai; ++k)
                    for (int i = 0; i < kWaitLimit && !mbar_try(&S.a_full[k % kAStages], (k / kAStages) & 1); ++i) {}
                for (unsigned k = bi > kBStages ? bi - kBStages : 0; k < bi; ++k)
                    for (int i = 0; i < kWaitLimit && !mbar_try(&S.b_full[k % kBStages], (k / kBStages) & 1); ++i) {}
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer: per item, segments of kSegChunks K chunks, each into
        // the next of two accumulator buffers
        if (lane == 0) {
            const uint32_t idesc = mma_idesc(N);
            unsigned ai = 0, bi = 0, seg = 0;
            bool ok = true;
            for (int it = it0; it < it1 && ok; ++it) {
                const PfColItem I = A.col_items[it];
                if (it + 2 < it1) prefetch_l1(A.col_items + it + 2);
                for (int kc0 = 0; kc0 < I.nkc && ok; kc0 += kSegChunks, ++seg) {
                    const int buf = seg & 1;
                    if (seg >= 2) ok = wait_bar(&S.acc_empty[buf], ((seg >> 1) - 1) & 1, abort_flag, status);
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t d = tmem + uint32_t(buf * kAccStride);
                    int acc = 0;
                    for (int kc = kc0; kc < min(I.nkc, kc0 + kSegChunks) && ok; ++kc) {
                        const int sb = bi % kBStages;
                        ok = wait_bar(&S.b_full[sb], (bi / kBStages) & 1, abort_flag, status);
                        if (!ok) break;
                        const uint32_t b_addr = smem_u32(sm + kOffBF16 + sb * kBTileBytes);
                        for (int m = 0; m < I.planes; ++m) {
                            const int sa = ai % kAStages;
                            ok = wait_bar(&S.a_conv[sa], (ai / kAStages) & 1, abort_flag, status);
                            if (!ok) break;
                            tc_fence_after();
                            const uint32_t a_addr = smem_u32(sm + kOffAF16 + sa * kPfTileBytes);
#pragma unroll
                            for (int ks = 0; ks < 4; ++ks) {
                                mma_f16(d, sw128_desc(a_addr + 32 * ks), sw128_desc(b_addr + 32 * ks), idesc, acc);
                                acc = 1;
                            }
                            mma_commit(&S.a_empty[sa]);
                            ++ai;
                        }
                        mma_commit(&S.b_empty[sb]);
                        ++bi;
                    }
                    mma_commit(&S.acc_full[buf]);
                }
            }
            // every MMA issued has finished before tensor memory is freed
            mma_commit(&S.drain);
            for (int i = 0; i < kWaitLimit && !mbar_try(&S.drain, 0); ++i) {}
        }
    } else if (warp < kEpiWarp0) {
        // ---- converters: digit planes -> f16 A tiles
        const int ctid = tid - kConvWarp0 * 32;
        unsigned ai = 0;
        bool ok = true;
        for (int it = it0; it < it1 && ok; ++it) {
            const PfColItem I = A.col_items[it];
            if (it + 2 < it1) prefetch_l1(A.col_items + it + 2);
            for (int kc = 0; kc < I.nkc && ok; ++kc)
                for (int m = 0; m < I.planes; ++m) {
                    const int sa = ai % kAStages;
                    ok = wait_bar(&S.a_full[sa], (ai / kAStages) & 1, abort_flag, status);
                    if (!ok) break;
                    convert_plane<kConvWarps * 32>(sm + kOffARaw + sa * kPfPlaneBytes, sm + kOffAF16 + sa * kPfTileBytes,
                                                   m, I.planes, 0, 0, ctid);
                    fence_async_smem();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&S.a_conv[sa]);
                    ++ai;
                }
        }
    } else {
        // ---- epilogue: T summed over the item's segments in FP32 registers,
        // then u = s T 2^(24 + E_r - 1037) per component and column, in FP32
        // (u is stored as FP32; the FP64 pipe of this part would take ~20 us
        // per item for the same work)
        const int q = warp & 3, j = 32 * q + lane;
        unsigned seg = 0;
        bool ok = true;
        for (int it = it0; it < it1 && ok; ++it) {
            const PfColItem I = A.col_items[it];
            if (it + 2 < it1) prefetch_l1(A.col_items + it + 2);
            PfComp C{};
            if (j < I.count) C = A.comps[I.comp0 + j];
            const float sf = float(C.scale);
            float t[kPfMaxRhs];
#pragma unroll
            for (int r = 0; r < kPfMaxRhs; ++r) t[r] = 0.0f;
            for (int kc0 = 0; kc0 < I.nkc; kc0 += kSegChunks, ++seg) {
                const int buf = seg & 1;
                if (!(ok = wait_bar(&S.acc_full[buf], (seg >> 1) & 1, abort_flag, status))) break;
                tc_fence_after();
                const uint32_t base = tmem + (uint32_t(32 * q) << 16) + uint32_t(buf * kAccStride);
#pragma unroll
                for (int g = 0; g < kPfMaxRhs / 16; ++g) {
                    if (16 * g >= p) break;
                    float v0[16], v1[16], v2[16];
                    tmem_ld16(base + 48 * g, v0);
                    tmem_ld16(base + 48 * g + 16, v1);
                    tmem_ld16(base + 48 * g + 32, v2);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        // columns 3i, 3i+1, 3i+2 of the 48: the limbs of right-hand side 16g + i
                        const int c0 = 3 * i, c1 = 3 * i + 1, c2 = 3 * i + 2;
                        const float a0 = c0 < 16 ? v0[c0] : (c0 < 32 ? v1[c0 - 16] : v2[c0 - 32]);
                        const float a1 = c1 < 16 ? v0[c1] : (c1 < 32 ? v1[c1 - 16] : v2[c1 - 32]);
                        const float a2 = c2 < 16 ? v0[c2] : (c2 < 32 ? v1[c2 - 16] : v2[c2 - 32]);
                        t[16 * g + i] += (a0 + a1) + a2;
                    }
                }
                // accumulator drained: release it to the MMA warp
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.acc_empty[buf]);
            }
            if (!ok) break;
#pragma unroll
            for (int g = 0; g < kPfMaxRhs / 16; ++g) {
                if (16 * g >= p) break;
                float u[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int r = 16 * g + i;
                    u[i] = (j < I.count && r < p) ? t[r] * sf * S.fxscale[r] : 0.0f;
                }
                for (int d = 0; d < (j < I.count ? C.ndest : 0); ++d) {
                    const int slot = __ldg(A.dests + C.dest0 + d) & 0x0FFFFFFF;
                    float4* dst = reinterpret_cast<float4*>(W.ut + (long long)slot * pu + 16 * g);
#pragma unroll
                    for (int k = 0; k < 4; ++k) dst[k] = make_float4(u[4 * k], u[4 * k + 1], u[4 * k + 2], u[4 * k + 3]);
                }
            }
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_free(tmem, 512);
}

// ------------------------------------------------------------ row kernel

template <int kSegChunks>
__global__ void __launch_bounds__(RowRoles::kThreads, 1) pf_row_kernel(Arena A, Work W,
                                                                       const __grid_constant__ CUtensorMap xmap, int p,
                                                                       int N, int pu, int u_beta, int* status) {
    constexpr int kConvWarps = RowRoles::kConvWarps, kEpiWarp0 = RowRoles::kEpiWarp0, kAStages = RowRoles::kAStages;
    constexpr int kOffAF16 = SmemMap<RowRoles>::kOffAF16, kOffBF16 = SmemMap<RowRoles>::kOffBF16,
                  kOffARaw = SmemMap<RowRoles>::kOffARaw, kOffBRaw = SmemMap<RowRoles>::kOffBRaw;
    extern __shared__ uint8_t smem_dyn[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
    __shared__ Shared S;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int it0 = __ldg(A.row_sched + blockIdx.x), it1 = __ldg(A.row_sched + blockIdx.x + 1);
    if (tid == 0) {
        init_barriers(S, kAStages, kConvWarps);
        S.abort_flag = 0;
    }
    if (tid < kPfMaxRhs) {
        const int E = tid < p ? W.ex[tid] : 0;
        S.ex[tid] = E;
        S.fdscale[tid] = E ? ldexpf(1.0f, max(-126, min(127, E - 1037))) : 0.0f;
        // U' = u 256^(P-1) 2^k < 2^15 by the layout-time bound
        // |u| 256^(P-1) < 2^(u_beta + E - 1022); an item applies its own,
        // smaller bound: k + (u_beta - the item's u_beta)
        S.ku[tid] = E ? 1037 - E - u_beta : kZeroColumn;
    }
    // B rows 3p .. N-1 of both f16 B stages stay zero (the converters write
    // only rows < 3p; tensor copies of x write zeros there)
    for (int idx = tid; idx < kBStages * (N - 3 * p) * 8; idx += RowRoles::kThreads) {
        const int s = idx / ((N - 3 * p) * 8), rest = idx % ((N - 3 * p) * 8);
        const int row = 3 * p + rest / 8, c = rest % 8;
        *reinterpret_cast<uint4*>(sm + kOffBF16 + s * kBTileBytes + swz_chunk(row, c)) = make_uint4(0u, 0u, 0u, 0u);
    }
    fence_async_smem();
    if (warp == 1) tmem_alloc(&S.tmem, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    volatile int* abort_flag = &S.abort_flag;

    if (warp == 0) {
        if (lane == 0) {
            unsigned ai = 0, bi = 0;
            bool ok = true;
            for (int it = it0; it < it1 && ok; ++it) {
                const PfRowItem I = A.row_items[it];
                for (int c = 0; c < I.nchunks && ok; ++c) {
                    const PfRowChunk C = A.chunks[I.chunk0 + c];
                    if (c + 2 < I.nchunks) prefetch_l1(A.chunks + I.chunk0 + c + 2);
                    const int sb = bi % kBStages;
                    if (bi >= kBStages) ok = wait_bar(&S.b_empty[sb], ((bi / kBStages) - 1) & 1, abort_flag, status);
                    if (!ok) break;
                    if (C.kind == 0) {
                        const unsigned bytes = unsigned(kPfK * pu * 4);
                        mbar_expect(&S.b_full[sb], bytes);
                        bulk_g2s(sm + kOffBRaw + sb * kURawBytes, W.ut + (long long)C.b * pu, bytes, &S.b_full[sb]);
                    } else {
                        mbar_expect(&S.b_full[sb], unsigned(N * 128));
                        tma_2d(sm + kOffBF16 + sb * kBTileBytes, &xmap, C.b, 0, &S.b_full[sb]);
                    }
                    ++bi;
                    const int nt = C.kind == 0 ? C.planes : 3;
                    const unsigned pbytes = C.kind == 0 ? unsigned((C.half == 0 ? 128 : 64) * kPfK) : unsigned(kPfTileBytes);
                    for (int m = 0; m < nt; ++m) {
                        const int sa = ai % kAStages;
                        if (ai >= kAStages) ok = wait_bar(&S.a_empty[sa], ((ai / kAStages) - 1) & 1, abort_flag, status);
                        if (!ok) break;
                        mbar_expect(&S.a_full[sa], pbytes);
                        uint8_t* dst = C.kind == 0 ? sm + kOffARaw + sa * kPfPlaneBytes : sm + kOffAF16 + sa * kPfTileBytes;
                        bulk_g2s(dst, A.praw + C.a_off + (long long)m * pbytes, pbytes, &S.a_full[sa]);
                        ++ai;
                    }
                }
            }
            if (!ok) {
                for (unsigned k = ai > kAStages ? ai - kAStages : 0; k < ai; ++k)
                    for (int i = 0; i < kWaitLimit && !mbar_try(&S.a_full[k % kAStages], (k / kAStages) & 1); ++i) {}
                for (unsigned k = bi > kBStages ? bi - kBStages : 0; k < bi; ++k)
                    for (int i = 0; i < kWaitLimit && !mbar_try(&S.b_full[k % kBStages], (k / kBStages) & 1); ++i) {}
            }
        }
    } else if (warp == 1) {
        // ---- MMA issuer: per item, segments of up to kSegChunks chunks of one
        // kind (low rank or dense), each into the next of two buffers
        if (lane == 0) {
            const uint32_t idesc = mma_idesc(N);
            unsigned ai = 0, bi = 0, seg = 0;
            bool ok = true;
            for (int it = it0; it < it1 && ok; ++it) {
                const PfRowItem I = A.row_items[it];
                int c = 0;
                while (c < I.nchunks && ok) {
                    const int kind = A.chunks[I.chunk0 + c].kind;
                    int c_end = c + 1;
                    while (c_end < I.nchunks && c_end - c < kSegChunks && A.chunks[I.chunk0 + c_end].kind == kind)
                        ++c_end;
                    const int buf = seg & 1;
                    if (seg >= 2) ok = wait_bar(&S.acc_empty[buf], ((seg >> 1) - 1) & 1, abort_flag, status);
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t d = tmem + uint32_t(buf * kAccStride);
                    int acc = 0;
                    for (; c < c_end && ok; ++c) {
                        const PfRowChunk C = A.chunks[I.chunk0 + c];
                        if (c + 2 < I.nchunks) prefetch_l1(A.chunks + I.chunk0 + c + 2);
                        const int sb = bi % kBStages;
                        ok = wait_bar(&S.b_conv[sb], (bi / kBStages) & 1, abort_flag, status);
                        if (!ok) break;
                        const uint32_t b_addr = smem_u32(sm + kOffBF16 + sb * kBTileBytes);
                        const int nt = C.kind == 0 ? C.planes : 3;
                        for (int m = 0; m < nt; ++m) {
                            const int sa = ai % kAStages;
                            ok = wait_bar(&S.a_conv[sa], (ai / kAStages) & 1, abort_flag, status);
                            if (!ok) break;
                            tc_fence_after();
                            const uint32_t a_addr = smem_u32(sm + kOffAF16 + sa * kPfTileBytes);
#pragma unroll
                            for (int ks = 0; ks < 4; ++ks) {
                                mma_f16(d, sw128_desc(a_addr + 32 * ks), sw128_desc(b_addr + 32 * ks), idesc, acc);
                                acc = 1;
                            }
                            mma_commit(&S.a_empty[sa]);
                            ++ai;
                        }
                        mma_commit(&S.b_empty[sb]);
                        ++bi;
                    }
                    mma_commit(&S.acc_full[buf]);
                    ++seg;
                }
            }
            mma_commit(&S.drain);
            for (int i = 0; i < kWaitLimit && !mbar_try(&S.drain, 0); ++i) {}
        }
    } else if (warp < kEpiWarp0) {
        const int ctid = tid - kConvWarp0 * 32;
        unsigned ai = 0, bi = 0;
        bool ok = true;
        for (int it = it0; it < it1 && ok; ++it) {
            const PfRowItem I = A.row_items[it];
            for (int c = 0; c < I.nchunks && ok; ++c) {
                const PfRowChunk C = A.chunks[I.chunk0 + c];
                if (c + 2 < I.nchunks) prefetch_l1(A.chunks + I.chunk0 + c + 2);
                const int sb = bi % kBStages;
                ok = wait_bar(&S.b_full[sb], (bi / kBStages) & 1, abort_flag, status);
                if (!ok) break;
                if (C.kind == 0)
                    convert_u<kConvWarps * 32>(reinterpret_cast<const float*>(sm + kOffBRaw + sb * kURawBytes),
                                               sm + kOffBF16 + sb * kBTileBytes, p, pu, C.nvalid, C.planes, S.ku,
                                               u_beta - I.u_beta, ctid);
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.b_conv[sb]);
                ++bi;
                const int nt = C.kind == 0 ? C.planes : 3;
                for (int m = 0; m < nt; ++m) {
                    const int sa = ai % kAStages;
                    ok = wait_bar(&S.a_full[sa], (ai / kAStages) & 1, abort_flag, status);
                    if (!ok) break;
                    if (C.kind == 0)
                        convert_plane<kConvWarps * 32>(sm + kOffARaw + sa * kPfPlaneBytes,
                                                       sm + kOffAF16 + sa * kPfTileBytes, m, C.planes,
                                                       24 - 8 * (C.planes - 1), C.half, ctid);
                    fence_async_smem();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&S.a_conv[sa]);
                    ++ai;
                }
            }
        }
    } else {
        // ---- epilogue: each segment's sums, scaled (2^-ku for low rank,
        // 2^(dense_exp + E_r - 1037) for dense), added into FP32 sums kept in
        // tensor memory (columns 192..255, which no MMA writes: N <= 192 and
        // the second accumulator starts at 256); the item's partial y stored
        // in FP64
        const int q = warp & 3, j = 32 * q + lane;
        const uint32_t yb = tmem + (uint32_t(32 * q) << 16) + 192u;
        unsigned seg = 0;
        bool ok = true;
        for (int it = it0; it < it1 && ok; ++it) {
            const PfRowItem I = A.row_items[it];
            {
                float z[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) z[i] = 0.0f;
#pragma unroll
                for (int g = 0; g < kPfMaxRhs / 16; ++g)
                    if (16 * g < p) tmem_st16(yb + 16 * g, z);
                tmem_wait_st();
                // this item's low-rank scales 2^-(ku + u_beta - item's u_beta)
                for (int r = lane; r < kPfMaxRhs; r += 32)
                    S.flitem[q][r] = S.ku[r] == kZeroColumn ? 0.0f : pow2f_clamped(-(S.ku[r] + u_beta - I.u_beta));
                __syncwarp();
            }
            const float dexp = ldexpf(1.0f, max(-126, min(127, I.dense_exp)));
            int c = 0;
            while (c < I.nchunks) {
                const int kind = A.chunks[I.chunk0 + c].kind;
                int c_end = c + 1;
                while (c_end < I.nchunks && c_end - c < kSegChunks && A.chunks[I.chunk0 + c_end].kind == kind) ++c_end;
                c = c_end;
                const int buf = seg & 1;
                if (!(ok = wait_bar(&S.acc_full[buf], (seg >> 1) & 1, abort_flag, status))) break;
                ++seg;
                tc_fence_after();
                const uint32_t base = tmem + (uint32_t(32 * q) << 16) + uint32_t(buf * kAccStride);
#pragma unroll 1
                for (int g = 0; g < kPfMaxRhs / 16; ++g) {
                    if (16 * g >= p) break;
                    float v0[16], v1[16], v2[16], y[16];
                    tmem_ld16(base + 48 * g, v0);
                    tmem_ld16(base + 48 * g + 16, v1);
                    tmem_ld16(base + 48 * g + 32, v2);
                    tmem_ld16(yb + 16 * g, y);
                    tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int r = 16 * g + i;
                        const int c0 = 3 * i, c1 = 3 * i + 1, c2 = 3 * i + 2;
                        const float a0 = c0 < 16 ? v0[c0] : (c0 < 32 ? v1[c0 - 16] : v2[c0 - 32]);
                        const float a1 = c1 < 16 ? v0[c1] : (c1 < 32 ? v1[c1 - 16] : v2[c1 - 32]);
                        const float a2 = c2 < 16 ? v0[c2] : (c2 < 32 ? v1[c2 - 16] : v2[c2 - 32]);
                        const float sc = kind == 0 ? S.flitem[q][r] : S.fdscale[r] * dexp;
                        y[i] = fmaf((a0 + a1) + a2, sc, y[i]);
                    }
                    tmem_st16(yb + 16 * g, y);
                }
                tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.acc_empty[buf]);
            }
            if (!ok) break;
            double* out = W.part + ((long long)I.part * kPfM + j) * pu;
#pragma unroll 1
            for (int g = 0; g < kPfMaxRhs / 16; ++g) {
                if (16 * g >= p) break;
                float y[16];
                tmem_ld16(yb + 16 * g, y);
                tmem_wait_ld();
                if (j < I.rows) {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (16 * g + i < p) out[16 * g + i] = double(y[i]);
                }
            }
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_free(tmem, 512);
}

// dst[i] = src[i], i < n: one pass of wide, independent loads, so that x in
// the caller's host memory crosses the host link once at full width (the
// exponent and limb kernels then read the device copy).
__global__ void __launch_bounds__(256) pf_copy_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                                      size_t n) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const double a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

// y[perm[row] * ld + r] = the tile's partials, summed in K-split order.
__global__ void __launch_bounds__(256) pf_combine_kernel(const int32_t* __restrict__ perm,
                                                         const int32_t* __restrict__ tile_part0,
                                                         const double* __restrict__ part, double* __restrict__ y,
                                                         long long ld, int n, int p, int pu) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n * p) return;
    const int row = int(idx / p), r = int(idx % p);
    const int t = row / kPfM, j = row % kPfM;
    const int h0 = __ldg(tile_part0 + t), h1 = __ldg(tile_part0 + t + 1);
    double s = 0.0;
    for (int h = h0; h < h1; ++h) s += part[((long long)h * kPfM + j) * pu + r];
    y[(long long)__ldg(perm + row) * ld + r] = s;
}

}  // namespace pf
}  // namespace qhg

// ------------------------------------------------------------ host side

using namespace qhg;

struct qh_pmatrix {
    PfLayout L;
    int device = 0;
    int sms = 1;
    void* arena = nullptr;
    int32_t* tile_part0 = nullptr;
    pf::Arena A{};
    std::mutex mu;
    void* own_ws = nullptr;
    size_t own_ws_bytes = 0;
    // qh_pmatmul_host: its stream, status word, pinned staging (devices
    // that cannot reach pageable host memory) and whether the kernels may
    // read x and write y in the caller's memory directly
    cudaStream_t stream = nullptr;
    int* d_status = nullptr;
    int* h_status = nullptr;
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    int host_direct = -1;  // -1: not probed yet
    int seg = pf::kDefaultSegChunks;  // K chunks per accumulation segment (1 or 2)
    ~qh_pmatrix() {
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        if (arena) cudaFree(arena);
        if (tile_part0) cudaFree(tile_part0);
        if (own_ws) cudaFree(own_ws);
        if (d_status) cudaFree(d_status);
        if (h_status) cudaFreeHost(h_status);
        if (pinned) cudaFreeHost(pinned);
        if (stream) cudaStreamDestroy(stream);
        cudaSetDevice(prev);
    }
};

namespace {

struct Guard {
    int prev = -1;
    explicit Guard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~Guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int cuda_err(cudaError_t e, const char* what) { return set_error(QH_ECUDA, std::string(what) + ": " + cudaGetErrorString(e)); }

size_t a256(size_t v) { return (v + 255) & ~size_t(255); }

// Scratch layout of one pass of up to 64 right-hand sides.
struct PfPlan {
    size_t ex, xt, ut, part, total;
    int p, pu, N, n_ent;
};

PfPlan pf_plan(const PfLayout& L, size_t rhs) {
    PfPlan w{};
    w.p = int(std::min<size_t>(rhs, kPfMaxRhs));
    w.pu = (w.p + 15) / 16 * 16;
    w.N = (3 * w.p + 15) / 16 * 16;
    w.n_ent = int((L.order + 7) / 8 * 8);
    size_t off = 0;
    auto take = [&](size_t b) {
        const size_t o = off;
        off += a256(std::max<size_t>(b, 16));
        return o;
    };
    w.ex = take(4 * kPfMaxRhs);
    w.xt = take(2 * size_t(w.N) * size_t(w.n_ent));
    w.ut = take(4 * size_t(L.n_slots) * size_t(w.pu));
    w.part = take(8 * size_t(L.n_parts) * kPfM * size_t(w.pu));
    w.total = off;
    return w;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

int pf_pass(const qh_pmatrix* m, const double* x, double* y, int p, long long ld, void* ws, cudaStream_t s,
            int* status, void* const* ev) {
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(static_cast<cudaEvent_t>(ev[i]), s);
    };
    const PfLayout& L = m->L;
    const PfPlan P = pf_plan(L, size_t(p));
    auto* w = static_cast<uint8_t*>(ws);
    pf::Work W;
    W.ex = reinterpret_cast<int*>(w + P.ex);
    W.xt = reinterpret_cast<__half*>(w + P.xt);
    W.ut = reinterpret_cast<float*>(w + P.ut);
    W.part = reinterpret_cast<double*>(w + P.part);
    const int n = int(L.order);
    auto encode = encode_fn();
    if (!encode) return set_error(QH_ECUDA, "cuTensorMapEncodeTiled is not available");
    CUtensorMap map;
    const cuuint64_t dims[2] = {cuuint64_t(P.n_ent), cuuint64_t(P.N)};
    const cuuint64_t strides[1] = {cuuint64_t(P.n_ent) * 2};
    const cuuint32_t box[2] = {cuuint32_t(kPfK), cuuint32_t(P.N)};
    const cuuint32_t estr[2] = {1, 1};
    CUresult cr = encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, W.xt, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) return set_error(QH_ECUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(cr)) + ")");
    cudaError_t e = cudaMemsetAsync(w + P.ex, 0, P.xt - P.ex, s);  // ex
    if (e != cudaSuccess) return cuda_err(e, "cudaMemsetAsync");
    mark(0);
    pf::pf_xmax_kernel<<<(n + 255) / 256, 64, 0, s>>>(x, ld, n, p, W.ex, status);
    pf::pf_xlimbs_kernel<<<(P.n_ent + 255) / 256, 256, 0, s>>>(x, ld, n, p, P.n_ent, P.N, m->A.perm, W.ex, W.xt);
    mark(1);
    if (L.n_col_items > 0) {
        if (m->seg == 1)
            pf::pf_column_kernel<1><<<L.grid, pf::ColRoles::kThreads, pf::kSmemColumn, s>>>(m->A, W, map, p, P.N, P.pu,
                                                                                           status);
        else
            pf::pf_column_kernel<2><<<L.grid, pf::ColRoles::kThreads, pf::kSmemColumn, s>>>(m->A, W, map, p, P.N, P.pu,
                                                                                           status);
    }
    mark(2);
    if (m->seg == 1)
        pf::pf_row_kernel<1><<<L.grid, pf::RowRoles::kThreads, pf::kSmemRow, s>>>(m->A, W, map, p, P.N, P.pu, L.u_beta,
                                                                                  status);
    else
        pf::pf_row_kernel<2><<<L.grid, pf::RowRoles::kThreads, pf::kSmemRow, s>>>(m->A, W, map, p, P.N, P.pu, L.u_beta,
                                                                                  status);
    mark(3);
    const long long total = (long long)n * p;
    pf::pf_combine_kernel<<<unsigned((total + 255) / 256), 256, 0, s>>>(m->A.perm, m->tile_part0, W.part, y, ld, n,
                                                                         p, P.pu);
    mark(4);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(e, "CUDA kernel launch");
    return QH_OK;
}

template <class F>
int guarded_pf(F&& f) {
    try {
        return f();
    } catch (const std::invalid_argument& e) {
        return set_error(QH_EINVAL, e.what());
    } catch (const std::overflow_error& e) {
        return set_error(QH_EOVERFLOW, e.what());
    } catch (const std::bad_alloc&) {
        return set_error(QH_ERUNTIME, "out of host memory");
    } catch (const std::exception& e) {
        return set_error(QH_ERUNTIME, e.what());
    }
}

// Build the precision layout of a matrix for `device` and upload it.
int pf_upload(const HostMatrix& hm, int device, int grid, double row_items_per_cta, qh_pmatrix** out) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_err(e, "cudaGetDeviceCount");
    if (!count) return set_error(QH_ERUNTIME, "no CUDA device is available");
    if (device < 0 || device >= count) return set_error(QH_EINVAL, "invalid CUDA device ordinal");
    Guard g(device);
    int sms = 1, cc_major = 0, cc_minor = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, device);
    if (cc_major != 10 || cc_minor != 3) return set_error(QH_ERUNTIME, "the precision form needs an sm_103 (GB300) device");
    auto* m = new (std::nothrow) qh_pmatrix();
    if (!m) return set_error(QH_ERUNTIME, "out of host memory");
    m->device = device;
    m->sms = sms;
    m->L = build_pf_layout(hm, grid > 0 ? std::min(grid, sms) : sms, row_items_per_cta);
    e = cudaMalloc(&m->arena, m->L.sec.total);
    if (e == cudaSuccess) e = cudaMemcpy(m->arena, m->L.arena.data(), m->L.sec.total, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&m->tile_part0, 4 * m->L.tile_part0.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(m->tile_part0, m->L.tile_part0.data(), 4 * m->L.tile_part0.size(), cudaMemcpyHostToDevice);
    for (auto* k : {pf::pf_column_kernel<1>, pf::pf_column_kernel<2>})
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, pf::kSmemColumn);
    for (auto* k : {pf::pf_row_kernel<1>, pf::pf_row_kernel<2>})
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, pf::kSmemRow);
    if (e != cudaSuccess) {
        delete m;
        return cuda_err(e, "precision form upload");
    }
    std::vector<uint8_t>().swap(m->L.arena);
    const PfSections& S = m->L.sec;
    auto* b = static_cast<const uint8_t*>(m->arena);
    m->A.perm = reinterpret_cast<const int32_t*>(b + S.perm);
    m->A.col_items = reinterpret_cast<const PfColItem*>(b + S.col_items);
    m->A.comps = reinterpret_cast<const PfComp*>(b + S.comps);
    m->A.dests = reinterpret_cast<const int32_t*>(b + S.dests);
    m->A.row_items = reinterpret_cast<const PfRowItem*>(b + S.row_items);
    m->A.chunks = reinterpret_cast<const PfRowChunk*>(b + S.chunks);
    m->A.col_sched = reinterpret_cast<const int32_t*>(b + S.col_sched);
    m->A.row_sched = reinterpret_cast<const int32_t*>(b + S.row_sched);
    m->A.qraw = b + S.qraw;
    m->A.praw = b + S.praw;
    *out = m;
    return QH_OK;
}

}  // namespace

extern "C" {

int qh_pmatrix_from_qhmat(const void* bytes, size_t len, int device, qh_pmatrix** out) {
    if (!out) return set_error(QH_EINVAL, "output handle pointer is null");
    *out = nullptr;
    if (!bytes && len) return set_error(QH_EINVAL, "image pointer is null");
    return guarded_pf([&] {
        HostMatrix hm = parse_qhmat(static_cast<const uint8_t*>(bytes), len);
        return pf_upload(hm, device, 0, 0.0, out);
    });
}

int qh_pmatrix_from_batch(const void* const* images, const size_t* lens, size_t count, int device, int grid,
                          double row_items_per_cta, qh_pmatrix** out, uint64_t* offsets) {
    if (!out) return set_error(QH_EINVAL, "output handle pointer is null");
    *out = nullptr;
    if (!images || !lens || !count) return set_error(QH_EINVAL, "empty batch");
    return guarded_pf([&] {
        std::vector<HostMatrix> ms;
        ms.reserve(count);
        for (size_t k = 0; k < count; ++k) ms.push_back(parse_qhmat(static_cast<const uint8_t*>(images[k]), lens[k]));
        std::vector<uint64_t> off;
        HostMatrix S = concat_block_diagonal(ms, kPfM, off);
        std::vector<HostMatrix>().swap(ms);
        const int rc = pf_upload(S, device, grid, row_items_per_cta, out);
        if (rc == QH_OK && offsets)
            for (size_t k = 0; k < count; ++k) offsets[k] = off[k];
        return rc;
    });
}

void qh_pmatrix_destroy(qh_pmatrix* m) { delete m; }

int qh_qhmat_device_bytes(const void* bytes, size_t len, int sms, uint64_t* plain_bytes, uint64_t* precision_bytes) {
    if (!plain_bytes && !precision_bytes) return set_error(QH_EINVAL, "no output requested");
    if (!bytes && len) return set_error(QH_EINVAL, "image pointer is null");
    if (sms < 1) return set_error(QH_EINVAL, "the SM count must be positive");
    return guarded_pf([&] {
        HostMatrix hm = parse_qhmat(static_cast<const uint8_t*>(bytes), len);
        if (plain_bytes) *plain_bytes = uint64_t(build_layout(hm).sec.total);
        if (precision_bytes) *precision_bytes = uint64_t(build_pf_layout(hm, sms, 0.0).sec.total);
        return int(QH_OK);
    });
}

size_t qh_pworkspace_bytes(const qh_pmatrix* m, size_t rhs) {
    return m && rhs ? pf_plan(m->L, rhs).total : 0;
}

int qh_pmatrix_stats(const qh_pmatrix* m, qh_pstats* out) {
    if (!m || !out) return set_error(QH_EINVAL, "null argument");
    const PfLayout& L = m->L;
    out->order = L.order;
    out->components = uint64_t(L.n_comp);
    out->code_bytes = L.code_bytes;
    out->scale_bytes = L.scale_bytes;
    out->dense_bytes = L.dense_bytes;
    out->stored_q_bytes = L.stored_q;
    out->stored_p_bytes = L.stored_p;
    out->stored_dense_bytes = L.stored_dense;
    out->device_bytes = L.sec.total;
    out->col_items = uint64_t(L.n_col_items);
    out->row_items = uint64_t(L.n_row_items);
    out->row_slots = uint64_t(L.n_slots);
    out->mma_elements = L.mma_col + L.mma_row;
    out->mma_col_elements = L.mma_col;
    out->mma_row_elements = L.mma_row;
    out->launches_per_pass = 4 + (L.n_col_items > 0 ? 1 : 0);
    out->segment_chunks = uint64_t(m->seg);
    return QH_OK;
}

int qh_pmatrix_set_segment_chunks(qh_pmatrix* m, int chunks) {
    if (!m) return set_error(QH_EINVAL, "null matrix handle");
    if (chunks != 1 && chunks != 2) return set_error(QH_EINVAL, "segment chunks must be 1 or 2");
    std::lock_guard<std::mutex> lock(m->mu);
    m->seg = chunks;
    return QH_OK;
}

int qh_pmatmul_device(const qh_pmatrix* m, const double* x, double* y, size_t rhs, void* workspace,
                      size_t workspace_bytes, void* stream, int* status) {
    return qh_pmatmul_device_profiled(m, x, y, rhs, workspace, workspace_bytes, stream, status, nullptr);
}

int qh_pmatmul_device_profiled(const qh_pmatrix* m, const double* x, double* y, size_t rhs, void* workspace,
                               size_t workspace_bytes, void* stream, int* status, void* const* events5) {
    if (!m) return set_error(QH_EINVAL, "null matrix handle");
    if (rhs == 0 || rhs > SIZE_MAX / m->L.order) return set_error(QH_EINVAL, "right-hand-side shape mismatch");
    if (m->L.order * rhs > size_t(INT32_MAX) * 256) return set_error(QH_EOVERFLOW, "CUDA launch grid too large");
    if (!x || !y) return set_error(QH_EINVAL, "null right-hand side or result pointer");
    Guard g(m->device);
    const size_t need = pf_plan(m->L, rhs).total;
    void* ws = workspace;
    auto* mm = const_cast<qh_pmatrix*>(m);
    std::unique_lock<std::mutex> lock(mm->mu, std::defer_lock);
    if (ws) {
        if (workspace_bytes < need) return set_error(QH_EINVAL, "workspace too small");
        if (reinterpret_cast<uintptr_t>(ws) & 255) return set_error(QH_EINVAL, "workspace must be 256-byte aligned");
    } else {
        lock.lock();
        if (mm->own_ws_bytes < need) {
            if (mm->own_ws) cudaFree(mm->own_ws);
            mm->own_ws = nullptr;
            mm->own_ws_bytes = 0;
            cudaError_t e = cudaMalloc(&mm->own_ws, need);
            if (e != cudaSuccess) return cuda_err(e, "cudaMalloc");
            mm->own_ws_bytes = need;
        }
        ws = mm->own_ws;
    }
    for (size_t c0 = 0; c0 < rhs; c0 += kPfMaxRhs) {
        const int p = int(std::min<size_t>(kPfMaxRhs, rhs - c0));
        const int rc = pf_pass(m, x + c0, y + c0, p, (long long)rhs, ws, static_cast<cudaStream_t>(stream), status,
                               c0 == 0 ? events5 : nullptr);
        if (rc) return rc;
    }
    return QH_OK;
}


int qh_pmatmul_host(const qh_pmatrix* m, const double* x, double* y, size_t rhs) {
    if (!m) return set_error(QH_EINVAL, "null matrix handle");
    if (rhs == 0 || rhs > SIZE_MAX / m->L.order / sizeof(double))
        return set_error(QH_EINVAL, "right-hand-side shape mismatch");
    if (m->L.order * rhs > size_t(INT32_MAX) * 256) return set_error(QH_EOVERFLOW, "CUDA launch grid too large");
    if (!x || !y) return set_error(QH_EINVAL, "null right-hand side or result pointer");
    Guard g(m->device);
    auto* mm = const_cast<qh_pmatrix*>(m);
    std::lock_guard<std::mutex> lock(mm->mu);
    cudaError_t e;
    if (mm->host_direct < 0) {
        int pageable = 0, host_tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, m->device);
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, m->device);
        mm->host_direct = pageable == 1 && host_tables == 1 ? 1 : 0;
    }
    if (!mm->stream && (e = cudaStreamCreateWithFlags(&mm->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_err(e, "cudaStreamCreate");
    if (!mm->d_status) {
        if ((e = cudaMalloc(&mm->d_status, sizeof(int))) != cudaSuccess) return cuda_err(e, "cudaMalloc");
        if ((e = cudaMallocHost(&mm->h_status, sizeof(int))) != cudaSuccess) return cuda_err(e, "cudaMallocHost");
    }
    const size_t vec = m->L.order * rhs * sizeof(double);
    const size_t need_ws = pf_plan(m->L, rhs).total;
    const auto* xb = reinterpret_cast<const uint8_t*>(x);
    const auto* yb = reinterpret_cast<const uint8_t*>(y);
    const bool direct = mm->host_direct == 1 && (xb + vec <= yb || yb + vec <= xb);
    // device buffer: workspace | x [| y when staged]
    const size_t need = a256(need_ws) + (direct ? a256(vec) : 2 * a256(vec));
    if (mm->own_ws_bytes < need) {
        if (mm->own_ws) cudaFree(mm->own_ws);
        mm->own_ws = nullptr;
        mm->own_ws_bytes = 0;
        if ((e = cudaMalloc(&mm->own_ws, need)) != cudaSuccess) return cuda_err(e, "cudaMalloc");
        mm->own_ws_bytes = need;
    }
    auto* base = static_cast<uint8_t*>(mm->own_ws);
    const double* dx = x;
    double* dy = y;
    if (direct) {
        // one write per page of y makes every page present and writable before
        // the device writes it
        static const uintptr_t page = uintptr_t(sysconf(_SC_PAGESIZE) > 0 ? sysconf(_SC_PAGESIZE) : 4096);
        const uintptr_t y0 = reinterpret_cast<uintptr_t>(y), y1 = y0 + vec;
        for (uintptr_t a = y0; a < y1; a = (a & ~(page - 1)) + page) *reinterpret_cast<volatile uint8_t*>(a) = 0;
        // x: one device copy, read across the host link once
        double* sx = reinterpret_cast<double*>(base + a256(need_ws));
        const size_t nx = m->L.order * rhs;
        const unsigned blocks = unsigned(std::min<size_t>((nx + 255) / 256, size_t(m->sms) * 8));
        pf::pf_copy_kernel<<<std::max(1u, blocks), 256, 0, mm->stream>>>(x, sx, nx);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e, "CUDA kernel launch");
        dx = sx;
    } else {
        if (mm->pinned_bytes < vec) {
            if (mm->pinned) cudaFreeHost(mm->pinned);
            mm->pinned = nullptr;
            mm->pinned_bytes = 0;
            if ((e = cudaMallocHost(&mm->pinned, vec)) != cudaSuccess) return cuda_err(e, "cudaMallocHost");
            mm->pinned_bytes = vec;
        }
        double* sx = reinterpret_cast<double*>(base + a256(need_ws));
        dy = reinterpret_cast<double*>(base + a256(need_ws) + a256(vec));
        dx = sx;
        std::memcpy(mm->pinned, x, vec);
        if ((e = cudaMemcpyAsync(sx, mm->pinned, vec, cudaMemcpyHostToDevice, mm->stream)) != cudaSuccess)
            return cuda_err(e, "cudaMemcpy host-to-device");
    }
    if ((e = cudaMemsetAsync(mm->d_status, 0, sizeof(int), mm->stream)) != cudaSuccess)
        return cuda_err(e, "cudaMemsetAsync");
    for (size_t c0 = 0; c0 < rhs; c0 += kPfMaxRhs) {
        const int p = int(std::min<size_t>(kPfMaxRhs, rhs - c0));
        const int rc = pf_pass(m, dx + c0, dy + c0, p, (long long)rhs, base, mm->stream, mm->d_status, nullptr);
        if (rc) return rc;
    }
    if (!direct && (e = cudaMemcpyAsync(mm->pinned, dy, vec, cudaMemcpyDeviceToHost, mm->stream)) != cudaSuccess)
        return cuda_err(e, "cudaMemcpy device-to-host");
    if ((e = cudaMemcpyAsync(mm->h_status, mm->d_status, sizeof(int), cudaMemcpyDeviceToHost, mm->stream)) !=
        cudaSuccess)
        return cuda_err(e, "cudaMemcpy device-to-host");
    if ((e = cudaStreamSynchronize(mm->stream)) != cudaSuccess) return cuda_err(e, "CUDA kernel execution");
    if (*mm->h_status & QH_STATUS_NONFINITE) return set_error(QH_EINVAL, "nonfinite right-hand side");
    if (*mm->h_status & QH_STATUS_TIMEOUT) return set_error(QH_ERUNTIME, "device copy wait timed out");
    if (!direct) std::memcpy(y, mm->pinned, vec);
    return QH_OK;
}

int qh_pmatrix_host_direct(const qh_pmatrix* m) {
    if (!m) return set_error(QH_EINVAL, "null matrix handle");
    int pageable = 0, host_tables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, m->device);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, m->device);
    return pageable == 1 && host_tables == 1 ? 1 : 0;
}

}  // extern "C"
