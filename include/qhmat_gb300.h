/*
 * qhmat_gb300 -- C ABI of the GB300-resident quantized H-matrix matvec.
 *
 * Plain C types only (pointers, sizes, ints); no torch or C++ types cross this
 * boundary.  Every entry point returns an int status (QH_OK on success) and
 * records a message for the calling thread, read back with qh_last_error().
 * Status codes map onto the exception types the reference raises through
 * pybind11: QH_EINVAL -> ValueError (std::invalid_argument), QH_ERUNTIME and
 * QH_ECUDA -> RuntimeError (std::runtime_error), QH_EOVERFLOW -> OverflowError
 * (std::overflow_error).
 *
 * What each entry replaces in inEXASCALE/qhmat:
 *   qh_matrix_from_qhmat  HMatrix::load (src/qhmat/io.cpp:173-257) plus the
 *                         per-call flatten + upload of HMatrix::matmul_cuda
 *                         (src/qhmat/cuda.cu:119-150), done once.
 *   qh_matrix_from_arrays the flattened arrays HMatrix::matmul_cuda builds on
 *                         every call (src/qhmat/cuda.cu:119-141), handed over
 *                         once; DeviceBlock (src/qhmat/cuda.cu:42-46) is
 *                         qh_block_desc below.
 *   qh_matmul_host        std::vector<double> HMatrix::matmul_cuda(x, rhs)
 *                         (src/qhmat/core.hpp:64-65, src/qhmat/cuda.cu:106-164):
 *                         host x in, host y out, same validation and messages.
 *   qh_matmul_device      the device-resident form of the same apply: x and y
 *                         are device pointers, stream-ordered, no host sync.
 *   qh_cuda_built         the module attribute qhmat.cuda_built
 *                         (src/qhmat/bindings.cpp:200-204).
 *
 * Layout of x and y (both entries): row-major order x rhs in SOURCE index
 * order, x[i*rhs + p], exactly as HMatrix::matmul takes and returns them
 * (src/qhmat/core.cpp:360-390).
 */
#ifndef QHMAT_GB300_H
#define QHMAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define QH_API __attribute__((visibility("default")))
#else
#define QH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define QH_OK 0
#define QH_EINVAL 1    /* ValueError    (std::invalid_argument in the reference) */
#define QH_ERUNTIME 2  /* RuntimeError  (std::runtime_error) */
#define QH_EOVERFLOW 3 /* OverflowError (std::overflow_error) */
#define QH_ECUDA 4     /* RuntimeError raised from a CUDA runtime failure */

/* Bits the device-side status int of qh_matmul_device / qh_matmul_device_static
 * may receive (OR-ed in; the call never clears it).  If either is set, y is
 * unspecified.  qh_matmul_host maps them to QH_EINVAL "nonfinite right-hand
 * side" and QH_ERUNTIME "device copy wait timed out". */
#define QH_STATUS_NONFINITE 1 /* x holds a NaN or an infinity */
#define QH_STATUS_TIMEOUT 2   /* a bounded device wait for a bulk copy gave up */

typedef struct qh_matrix qh_matrix;

/* Mirrors DeviceBlock (src/qhmat/cuda.cu:42-46): one block of the partition in
 * clustered coordinates.  factor_offset indexes the per-component arrays
 * (widths, scales, offsets); dense_offset indexes the dense value array. */
typedef struct {
    size_t row0, row1, col0, col1;
    size_t rank, factor_offset, dense_offset;
    int is_dense;
} qh_block_desc;

/* Size figures of a resident matrix (all in bytes unless named otherwise).
 * model_bytes is the packed-byte traffic model of one single-RHS apply:
 * 4*(left+right code words) + 16*sum(rank) + 8*sum(dense m*n) + 16*order. */
typedef struct {
    uint64_t order, block_count, dense_blocks, lowrank_blocks, components;
    uint64_t code_bytes;      /* 4 * (left + right code words), as stored by the reference */
    uint64_t scale_bytes;     /* 16 * sum(rank): one left and one right FP64 scale each */
    uint64_t dense_bytes;     /* 8 * sum over dense blocks of m*n */
    uint64_t model_bytes;     /* code + scale + dense + 16*order (x read, y written) */
    uint64_t device_bytes;    /* bytes the resident layout occupies on the device */
    uint64_t row_tiles;       /* row-side work units */
    uint64_t flops_per_rhs;   /* 2*(sum rank*(m+n) + sum dense m*n) */
    uint64_t launches_per_apply; /* kernels one qh_matmul_device call launches */
    uint64_t host_direct;     /* 1: qh_matmul_host's kernels read x / write y in host memory */
    uint64_t left_code_bytes;  /* 4 * left (row-side, P) code words */
    uint64_t right_code_bytes; /* 4 * right (column-side, Q) code words */
} qh_stats;

/* Message of the last failing call made by this thread ("" if none). */
QH_API const char* qh_last_error(void);

/* 1: this library applies on CUDA devices (mirrors qhmat.cuda_built). */
QH_API int qh_cuda_built(void);

/* Parse and validate a QHMAT001 image with the reference's checks and
 * messages, build the resident layout, and upload it to `device` (one
 * cudaMalloc'd arena owned by the handle). */
QH_API int qh_matrix_from_qhmat(const void* bytes, size_t len, int device, qh_matrix** out);

/* Same, from the arrays HMatrix::matmul_cuda flattens (cuda.cu:119-141):
 * permutation[order]; blocks[block_count]; dense values concatenated in block
 * order; left/right words concatenated in block order with per-component
 * offsets already rebased onto those arrays; scales and widths per component.
 * The partition is validated as HMatrix::finalize does (core.cpp:332-358). */
QH_API int qh_matrix_from_arrays(size_t order, const size_t* permutation, size_t block_count,
                          const qh_block_desc* blocks, const double* dense,
                          const uint32_t* left_words, const uint32_t* right_words,
                          const size_t* left_offsets, const size_t* right_offsets,
                          const double* left_scales, const double* right_scales,
                          const int* widths, int device, qh_matrix** out);

QH_API void qh_matrix_destroy(qh_matrix* m);

QH_API int qh_matrix_stats(const qh_matrix* m, qh_stats* out);

/* Max-norm bound of the stored matrix (HMatrix::reconstruction_bound,
 * src/qhmat/core.cpp:467-472). */
QH_API double qh_matrix_reconstruction_bound(const qh_matrix* m);

/* Device scratch (bytes) one qh_matmul_device call with `rhs` columns needs
 * (applies with more than 65535 columns run in column chunks of 65535 that
 * share one chunk's scratch). */
QH_API size_t qh_workspace_bytes(const qh_matrix* m, size_t rhs);

/* y = A x on the device.  x, y: device pointers, row-major order x rhs, source
 * order.  workspace: device scratch of at least qh_workspace_bytes(m, rhs)
 * bytes, 256-byte aligned, not shared with a concurrent call; NULL uses a
 * buffer the handle allocates on first use (shared by all NULL-workspace
 * calls on the handle, which must therefore not overlap on the GPU; separate
 * from qh_matmul_host's buffers).  stream: a cudaStream_t (NULL =
 * legacy default stream).  status: optional device int into which the call
 * ORs QH_STATUS_NONFINITE (x holds a NaN or infinity) and QH_STATUS_TIMEOUT
 * (a bounded device wait gave up); it is left untouched otherwise, and y is
 * unspecified if either bit is set.  Errors before any device work follow the
 * reference (src/qhmat/cuda.cu:108-112): rhs == 0 -> QH_EINVAL
 * "right-hand-side shape mismatch", order * rhs > INT_MAX * 256 ->
 * QH_EOVERFLOW "CUDA launch grid too large".  Stream-ordered: returns once
 * the work is enqueued. */
QH_API int qh_matmul_device(const qh_matrix* m, const double* x, double* y, size_t rhs,
                     void* workspace, size_t workspace_bytes, void* stream, int* status);

/* qh_matmul_device that also records four caller-created cudaEvent_t on
 * `stream`: before the right-hand-side preparation kernel, before the
 * column-side kernel, before the row-side kernel, and after it.  Profiling
 * aid (per-kernel durations); the work done is identical. */
QH_API int qh_matmul_device_profiled(const qh_matrix* m, const double* x, double* y, size_t rhs,
                                     void* workspace, size_t workspace_bytes, void* stream,
                                     int* status, void* const* events4);

/* Bytes of the fixed device scratch array qh_matmul_device_static uses. */
#define QH_STATIC_SCRATCH_BYTES (16u << 20)

/* qh_matmul_device for callers that cannot allocate device memory during an
 * apply -- a plugin whose host framework owns all device memory through its
 * own allocator, a latency-critical loop that cannot afford cudaMalloc's
 * implicit device synchronisation, code held to a fixed pre-reserved memory
 * budget.  It allocates nothing: its scratch is a file-scope static
 * __device__ array of QH_STATIC_SCRATCH_BYTES (16 MiB) that every GPU which
 * loads this library holds until the process exits.  The caller still passes
 * x and y (device pointers, row-major order x rhs, source order), the stream
 * and the optional status int (QH_STATUS_* bits), as for qh_matmul_device.
 * An apply whose scratch (qh_workspace_bytes(m, rhs)) exceeds
 * QH_STATIC_SCRATCH_BYTES is rejected with QH_EINVAL.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and
 * caches it for the life of the process; make that first call before any
 * stream capture.  A cudaDeviceReset of that device invalidates the cached
 * address: do not call this entry point on a device after resetting it.  All
 * calls share the one array (each call clears the parts that must start at
 * zero), so calls that overlap on the GPU -- concurrent streams, or several
 * threads -- race and must be serialised by the caller.  No counterpart in
 * the reference. */
QH_API int qh_matmul_device_static(const qh_matrix* m, const double* x, double* y, size_t rhs,
                                   void* stream, int* status);

/* Drop-in for HMatrix::matmul_cuda: host x (order*rhs doubles), host y.
 * On a device that reads and writes pageable host memory through the host's
 * page tables (a coherent host link, as on Grace), the kernels read x and
 * write y in place; elsewhere, and when x and y overlap, x is copied in
 * through pinned staging and y copied back.  Synchronises before returning.
 * Raises the reference's errors: "right-hand-side shape mismatch",
 * "nonfinite right-hand side" (QH_EINVAL; y is then unspecified), "CUDA
 * launch grid too large" (QH_EOVERFLOW), "no CUDA device is available"
 * (QH_ERUNTIME). */
QH_API int qh_matmul_host(const qh_matrix* m, const double* x, double* y, size_t rhs);

/* FNV-1a-64 of a byte range, the QHMAT001 trailer checksum (offset basis
 * 14695981039346656037, prime 1099511628211; src/qhmat/io.cpp:18-19, 42).
 * Used when writing QHMAT001 images. */
QH_API uint64_t qh_fnv1a64(const void* bytes, size_t len);

/* Dense reconstruction of the represented matrix, the reference's
 * HMatrix::reconstruct (src/qhmat/core.cpp:392-410) behind HMatrix.to_dense
 * (python/qhmat/matrix.py:309-311, bindings.cpp:180-190), on the GPU: `out`
 * receives order x order doubles, row-major in source order (entry (i, k) at
 * out[i * order + k]); out_on_device != 0 if `out` is device memory.  The
 * entries equal the reference's bit for bit (same FP64 operations in the
 * same order).  Synchronises.  Errors: "output size does not match order *
 * order" (QH_EINVAL), "dense output size overflow" (QH_EOVERFLOW). */
QH_API int qh_matrix_reconstruct(const qh_matrix* m, double* out, size_t out_count, int out_on_device);

/* Validation aid: decode every stored code of one factor side on the device
 * with the same device routine the apply kernels use, and copy the integers
 * to host `out`, component-major in block order (component c of a block with
 * `rows` entries on that side fills rows consecutive ints).  side 0 = left /
 * P (block rows), side 1 = right / Q (block columns).  `out_count` must equal
 * the total number of codes on that side (returned through `needed` when out
 * is NULL).  No reference counterpart: it exposes HMatrix::decode
 * (src/qhmat/core.cpp:269-282) semantics of the resident layout for tests. */
QH_API int qh_debug_decode(const qh_matrix* m, int side, int32_t* out, size_t out_count,
                           size_t* needed);

/* ---- Precision form: many right-hand sides per code stream (tcgen05) ----
 *
 * The reference re-decodes every code once per right-hand-side column
 * (src/qhmat/core.cpp:377-386) and its CUDA path does the same per thread
 * (src/qhmat/cuda.cu:64-102).  A qh_pmatrix holds a second resident layout of
 * the same QHMAT001 image, built for the 5th-generation tensor cores: each
 * code digit is read once per pass of up to 64 right-hand sides and
 * multiplied, as an exact f16 operand, by the hi/mid/lo f16 limbs of all of
 * them (FP32 accumulation in tensor memory); the per-component FP64 scales,
 * the dense diagonal blocks (three f16 limbs against the x limbs) and the
 * final y sums are combined in FP64.  Results carry FP32-level rounding
 * (about 1e-7 relative to the partial sums), not the plain form's ~1e-15:
 * callers choose this form when that error fits their budget (the Python
 * layer's gate: max |y_pf - y_plain| per column below 1% of
 * reconstruction_bound * ||x||_1).  Needs an sm_103 device. */
typedef struct qh_pmatrix qh_pmatrix;

typedef struct {
    uint64_t order, components;
    uint64_t code_bytes, scale_bytes, dense_bytes; /* packed-byte model, as qh_stats */
    uint64_t stored_q_bytes, stored_p_bytes, stored_dense_bytes; /* digit planes and dense limb tiles */
    uint64_t device_bytes;
    uint64_t col_items, row_items, row_slots;
    uint64_t mma_elements;      /* M x K elements through the MMAs per pass (x N = 3p limbs) */
    uint64_t launches_per_pass; /* kernels per pass of <= 64 right-hand sides */
    uint64_t mma_col_elements, mma_row_elements; /* the column and row kernels' shares */
    uint64_t segment_chunks;    /* K chunks per FP32 accumulation segment (1 or 2) */
} qh_pstats;

/* Parse a QHMAT001 image (the checks and messages of qh_matrix_from_qhmat)
 * and upload the precision-form layout to `device`. */
QH_API int qh_pmatrix_from_qhmat(const void* bytes, size_t len, int device, qh_pmatrix** out);
/* Device bytes the resident arenas of a QHMAT001 image will take, without
 * touching a device: the plain form's (qh_stats.device_bytes of
 * qh_matrix_from_qhmat) and the precision form's (qh_pstats.device_bytes of
 * qh_pmatrix_from_qhmat on a device of `sms` multiprocessors, whose
 * schedules it sizes); either output may be NULL.  Parses the image with the
 * checks and messages of qh_matrix_from_qhmat.  For admission control before
 * an upload.  No reference counterpart. */
QH_API int qh_qhmat_device_bytes(const void* bytes, size_t len, int sms, uint64_t* plain_bytes,
                                 uint64_t* precision_bytes);
QH_API void qh_pmatrix_destroy(qh_pmatrix* m);
QH_API int qh_pmatrix_stats(const qh_pmatrix* m, qh_pstats* out);
/* K chunks (of 64 entries) that one FP32 accumulation segment spans: 2 (the
 * default) or 1.  The tensor cores truncate as they accumulate, so shorter
 * segments halve this form's error (2.4e-7 vs 4.8e-7 relative to the plain
 * form on an n=32768 x 64 apply) for ~4% more time per pass.  Set it before
 * applies, not during them.  No reference counterpart. */
QH_API int qh_pmatrix_set_segment_chunks(qh_pmatrix* m, int chunks);
/* Device scratch of one qh_pmatmul_device call with `rhs` columns (passes of
 * 64 columns share it). */
QH_API size_t qh_pworkspace_bytes(const qh_pmatrix* m, size_t rhs);
/* y = A x in the precision form: x, y device pointers, row-major order x rhs,
 * source order (as qh_matmul_device); workspace NULL = a handle-owned buffer
 * (calls must then not overlap on the GPU); status: QH_STATUS_* bits.
 * Stream-ordered.  Column chunks of 64 right-hand sides run in turn. */
QH_API int qh_pmatmul_device(const qh_pmatrix* m, const double* x, double* y, size_t rhs, void* workspace,
                             size_t workspace_bytes, void* stream, int* status);
/* The same, recording five caller-created cudaEvent_t around the first pass's
 * kernels: before the x preparation, before the column kernel, before the
 * row kernel, before the combine, after it.  Profiling aid. */
QH_API int qh_pmatmul_device_profiled(const qh_pmatrix* m, const double* x, double* y, size_t rhs,
                                      void* workspace, size_t workspace_bytes, void* stream, int* status,
                                      void* const* events5);

/* y = A x in the precision form with x and y in host memory (row-major
 * order x rhs, source order), as qh_matmul_host is for the plain form: on a
 * device that reaches pageable host memory through the host's page tables
 * (GB300 on its Grace host) the kernels read x and write y in the caller's
 * buffers directly, elsewhere they are staged through pinned memory with one
 * copy each way.  Synchronous; the checks and messages of qh_matmul_host.
 * The precision-form counterpart of the reference's matmul_cuda
 * (src/qhmat/cuda.cu:106-164) for many right-hand sides. */
QH_API int qh_pmatmul_host(const qh_pmatrix* m, const double* x, double* y, size_t rhs);
/* 1 when qh_pmatmul_host reads and writes host buffers in place on this
 * handle's device, 0 when it stages them. */
QH_API int qh_pmatrix_host_direct(const qh_pmatrix* m);

/* ---- Batched applies (serving): column gather / scatter ----
 *
 * The reference applies one request at a time and copies every operand per
 * call (src/qhmat/bindings.cpp:152-179, src/qhmat/cuda.cu:143-164).  A serving
 * loop here gathers the columns of many requests into one multi-column
 * operand, applies once, and scatters the result columns back:
 *   gather:  dst[i * ld_dst + j] = src[i * ld_src + cols[j]]
 *   scatter: dst[i * ld_dst + cols[j]] = src[i * ld_src + j]
 * for rows i < n and j < ncols.  src / dst may be device memory or pinned
 * host memory the device reads and writes directly; cols is a device (or
 * pinned host) array of ncols column indices.  Stream-ordered, no copies of
 * their own.  No reference counterpart. */
QH_API int qh_gather_columns(const double* src, long long ld_src, double* dst, long long ld_dst,
                             const int32_t* cols, int ncols, size_t n, void* stream);
QH_API int qh_scatter_columns(const double* src, long long ld_src, double* dst, long long ld_dst,
                              const int32_t* cols, int ncols, size_t n, void* stream);

/* ---- Batching form: many matrices in one launch chain ----
 *
 * The reference applies one matrix per call.  A batch here is the
 * block-diagonal matrix diag(A_1, .., A_M) of M QHMAT001 images (offsets[k]
 * receives matrix k's first row: consecutive for the plain form, each on a
 * multiple of 128 rows for the precision form), resident as one plain-form
 * handle (qh_matrix_from_batch) or one
 * precision-form handle (qh_pmatrix_from_batch, whose persistent schedule uses
 * `grid` CTAs (0: one per SM) and about `row_items_per_cta` row items per CTA
 * (0: 3) -- the parameters the batching form's autotuner sets).  One
 * qh_matmul_device / qh_pmatmul_device call on the handle then walks the
 * blocks of every matrix in one persistent launch of each kernel.
 *
 * Right-hand sides of different sizes are packed: matrix k's x (order_k x
 * rhs_k, row-major, source order) at x_all + x_offset, its y at y_all +
 * y_offset.  qh_batch_gather builds the block-diagonal operand xs ((sum of
 * padded orders) x P, P = the largest rhs_k) with every column of every
 * matrix scaled by a power of two so that its largest |x| is in [1, 2)
 * (exps receives the exponents, count x P ints of device scratch), zero in
 * padding rows and columns; qh_batch_scatter scales the result back into
 * y_all, exactly.  table: a device array of count entries.  No reference
 * counterpart. */
typedef struct {
    uint64_t offset;   /* first row of the matrix in the block-diagonal operand */
    uint64_t order;    /* its order */
    uint64_t rows;     /* rows up to the next matrix (order plus padding) */
    uint64_t rhs;      /* its right-hand-side columns */
    uint64_t x_offset; /* element offset of its x in x_all */
    uint64_t y_offset; /* element offset of its y in y_all */
} qh_batch_entry;

QH_API int qh_matrix_from_batch(const void* const* images, const size_t* lens, size_t count, int device,
                                qh_matrix** out, uint64_t* offsets);
QH_API int qh_pmatrix_from_batch(const void* const* images, const size_t* lens, size_t count, int device, int grid,
                                 double row_items_per_cta, qh_pmatrix** out, uint64_t* offsets);
QH_API int qh_batch_gather(const qh_batch_entry* table, size_t count, int P, const double* x_all, double* xs,
                           int* exps, void* stream);
QH_API int qh_batch_scatter(const qh_batch_entry* table, size_t count, int P, const double* ys, const int* exps,
                            double* y_all, void* stream);

/* Test aid for the bounded device waits: one warp on `device` waits at most
 * `polls` (1 .. 2^20) tests on an mbarrier that nothing completes -- no copy
 * is issued -- and records the timeout in a status int exactly as the apply
 * kernels do; returns QH_ERUNTIME "device copy wait timed out" when the bit
 * came back (the expected outcome), QH_OK if the wait unexpectedly succeeded.
 * No reference counterpart. */
QH_API int qh_debug_wait_timeout(int device, int polls);

#ifdef __cplusplus
}
#endif

#endif /* QHMAT_GB300_H */
