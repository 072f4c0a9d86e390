// Column gather / scatter for batched applies (serving and batching forms).
//
// A batch of requests for one matrix is applied as one multi-column apply:
// the requests' right-hand-side columns are gathered from wherever they live
// (device memory, or pinned host memory the device reads directly) into one
// row-major order x p operand, and the result columns are scattered back to
// each request's output.  One launch each way per batch, instead of one copy
// per request.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/qhmat_gb300.h"
#include "errors.hpp"

namespace qhg {
namespace {

// Thread per (row, column j of the batch): dst[i * ld_dst + j] =
// src[i * ld_src + cols[j]] (gather), or dst[i * ld_dst + cols[j]] =
// src[i * ld_src + j] (scatter).  Rows in blockIdx.y-strided chunks.
template <bool GATHER>
__global__ void __launch_bounds__(256) columns_kernel(const double* __restrict__ src, long long ld_src,
                                                      double* __restrict__ dst, long long ld_dst,
                                                      const int32_t* __restrict__ cols, int ncols, long long n) {
    const int j = threadIdx.x % 64 + blockIdx.x * 64;
    if (j >= ncols) return;
    const int c = __ldg(cols + j);
    for (long long i = blockIdx.y * 4 + threadIdx.x / 64; i < n; i += 4LL * gridDim.y) {
        if (GATHER)
            dst[i * ld_dst + j] = src[i * ld_src + c];
        else
            dst[i * ld_dst + c] = src[i * ld_src + j];
    }
}

int launch_columns(bool gather, const double* src, long long ld_src, double* dst, long long ld_dst,
                   const int32_t* cols, int ncols, size_t n, void* stream) {
    if (!src || !dst || !cols) return set_error(QH_EINVAL, "null pointer");
    if (ncols <= 0 || n == 0) return QH_OK;
    const unsigned gx = unsigned((ncols + 63) / 64);
    const unsigned gy = unsigned(n < 4 * 1024 ? (n + 3) / 4 : 1024);
    auto s = static_cast<cudaStream_t>(stream);
    if (gather)
        columns_kernel<true><<<dim3(gx, gy), 256, 0, s>>>(src, ld_src, dst, ld_dst, cols, ncols, (long long)n);
    else
        columns_kernel<false><<<dim3(gx, gy), 256, 0, s>>>(src, ld_src, dst, ld_dst, cols, ncols, (long long)n);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(QH_ECUDA, std::string("CUDA kernel launch: ") + cudaGetErrorString(e));
    return QH_OK;
}

// Largest exponent field of column r of matrix m's right-hand side (block
// (m, r), 256 threads); 0 past the matrix's columns or for a zero column.
__global__ void __launch_bounds__(256) batch_exp_kernel(const qh_batch_entry* __restrict__ tab, const double* __restrict__ x,
                                                        int P, int* __restrict__ exps) {
    const qh_batch_entry E = tab[blockIdx.x];
    const int r = blockIdx.y;
    int m = 0;
    if (r < int(E.rhs))
        for (uint64_t i = threadIdx.x; i < E.order; i += blockDim.x) {
            const int e = int((__double_as_longlong(x[E.x_offset + i * E.rhs + r]) >> 52) & 0x7FF);
            m = max(m, e == 0x7FF ? 0 : e);
        }
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    __shared__ int sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) m = max(m, sm[w]);
        exps[blockIdx.x * P + r] = m;
    }
}

// 2^k as a double for |k| <= 1022.
__device__ __forceinline__ double pow2(int k) { return __longlong_as_double((long long)(1023 + k) << 52); }

// Block (m, chunk): rows of matrix m's slab [offset, offset + padded rows) of
// the block-diagonal operand, P columns.  Gather: xs = x scaled by 2^(1023 -
// e(m, r)) (max |x| of each column in [1, 2); exact), zero in padding rows
// and columns.  Scatter: y = ys scaled back by 2^(e(m, r) - 1023).
template <bool GATHER>
__global__ void __launch_bounds__(256) batch_move_kernel(const qh_batch_entry* __restrict__ tab, const int* __restrict__ exps,
                                                         int P, const double* __restrict__ src, double* __restrict__ dst) {
    const qh_batch_entry E = tab[blockIdx.y];
    const uint64_t rows = GATHER ? E.rows : E.order;
    const uint64_t total = rows * uint64_t(P);
    for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t i = t / uint64_t(P);
        const int r = int(t % uint64_t(P));
        const int e = exps[blockIdx.y * P + r];
        if (GATHER) {
            double v = 0.0;
            if (i < E.order && r < int(E.rhs) && e) v = src[E.x_offset + i * E.rhs + r] * pow2(1023 - e);
            dst[(E.offset + i) * uint64_t(P) + r] = v;
        } else if (r < int(E.rhs)) {
            const double v = src[(E.offset + i) * uint64_t(P) + r];
            dst[E.y_offset + i * E.rhs + r] = e ? v * pow2(e - 1023) : 0.0;
        }
    }
}

}  // namespace
}  // namespace qhg

extern "C" {

int qh_batch_gather(const qh_batch_entry* table, size_t count, int P, const double* x_all, double* xs, int* exps,
                    void* stream) {
    if (!table || !x_all || !xs || !exps || !count || P <= 0) return qhg::set_error(QH_EINVAL, "invalid batch gather");
    auto s = static_cast<cudaStream_t>(stream);
    qhg::batch_exp_kernel<<<dim3(unsigned(count), unsigned(P)), 256, 0, s>>>(table, x_all, P, exps);
    qhg::batch_move_kernel<true><<<dim3(64, unsigned(count)), 256, 0, s>>>(table, exps, P, x_all, xs);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return qhg::set_error(QH_ECUDA, std::string("CUDA kernel launch: ") + cudaGetErrorString(e));
    return QH_OK;
}

int qh_batch_scatter(const qh_batch_entry* table, size_t count, int P, const double* ys, const int* exps,
                     double* y_all, void* stream) {
    if (!table || !y_all || !ys || !exps || !count || P <= 0) return qhg::set_error(QH_EINVAL, "invalid batch scatter");
    auto s = static_cast<cudaStream_t>(stream);
    qhg::batch_move_kernel<false><<<dim3(64, unsigned(count)), 256, 0, s>>>(table, exps, P, ys, y_all);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return qhg::set_error(QH_ECUDA, std::string("CUDA kernel launch: ") + cudaGetErrorString(e));
    return QH_OK;
}


int qh_gather_columns(const double* src, long long ld_src, double* dst, long long ld_dst, const int32_t* cols,
                      int ncols, size_t n, void* stream) {
    return qhg::launch_columns(true, src, ld_src, dst, ld_dst, cols, ncols, n, stream);
}

int qh_scatter_columns(const double* src, long long ld_src, double* dst, long long ld_dst, const int32_t* cols,
                       int ncols, size_t n, void* stream) {
    return qhg::launch_columns(false, src, ld_src, dst, ld_dst, cols, ncols, n, stream);
}

}  // extern "C"
