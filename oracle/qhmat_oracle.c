/*
 * qhmat oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU path for the quantized
 * H-matrix matvec, used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg as the checker.  The product (qhmat_gb300/) never links, loads
 * or calls anything here; the GPU path fails loudly when its CUDA library is
 * missing instead of falling back to this file.
 *
 * Parity is pinned: tests/test_oracle.py compares every function below
 * bit-for-bit with the reference's own core compiled from its sources
 * (oracle/_ref/libqhmat_ref.so, built by oracle/build_ref.py) and with the
 * golden fixtures in tests/golden/ produced by the reference's HMatrix.
 *
 * Reference functions restated (file:line within inEXASCALE/qhmat):
 *   qho_parse        HMatrix::load + Reader       src/qhmat/io.cpp:69-123, 173-257
 *                    HMatrix::HMatrix (bijection) src/qhmat/core.cpp:205-212
 *                    check_rectangle              src/qhmat/core.cpp:214-222
 *                    finalize (cover check)       src/qhmat/core.cpp:332-358
 *   decode_code      HMatrix::decode              src/qhmat/core.cpp:269-282
 *   qho_matmul       HMatrix::matmul              src/qhmat/core.cpp:360-390
 *   qho_reconstruct  HMatrix::reconstruct         src/qhmat/core.cpp:392-410
 *   qho_bound        reconstruction_bound         src/qhmat/core.cpp:467-472
 *   qho_pack         HMatrix::pack                src/qhmat/core.cpp:235-267
 *
 * qho_matmul may split the clustered rows over threads.  Every thread walks
 * the blocks in insertion order and applies, for the rows it owns, exactly the
 * reference's sequence of FP64 operations, recomputing a low-rank block's
 * column-side dot product when the block straddles two threads.  Each y entry
 * therefore sees the same operations in the same order as in the
 * single-threaded reference, so the result is bit-identical for any thread
 * count.
 */
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QHO_EXPORT __attribute__((visibility("default")))

typedef struct {
    uint64_t row0, row1, col0, col1;
    uint8_t admissible, dense;
    double* values; /* dense: (row1-row0) x (col1-col0), row-major */
    uint64_t rank, menu_size;
    double truncation_error, quantization_bound;
    uint8_t* widths;
    double *left_scales, *right_scales;
    uint32_t *left_words, *right_words;
    uint64_t *left_offsets, *right_offsets;
    uint64_t left_word_count, right_word_count;
} qho_block;

typedef struct {
    uint64_t order, block_count;
    uint64_t* permutation; /* clustered position -> source index */
    qho_block* blocks;
} qho_matrix;

static void set_err(char* err, size_t len, const char* fmt, ...) {
    if (!err || !len) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, len, fmt, ap);
    va_end(ap);
}

/* ---------------------------------------------------------------- reader */

typedef struct {
    const uint8_t* p;
    uint64_t remaining; /* bytes left including the 8-byte checksum */
    uint64_t hash;
    int failed;
    const char* why;
} reader;

static const uint64_t FNV_OFFSET = 14695981039346656037ULL; /* io.cpp:18 */
static const uint64_t FNV_PRIME = 1099511628211ULL;        /* io.cpp:19 */

static uint64_t remaining_data(const reader* r) { return r->remaining < 8 ? 0 : r->remaining - 8; }

static uint8_t rd_byte(reader* r) {
    if (r->failed) return 0;
    if (remaining_data(r) == 0) {
        r->failed = 1;
        r->why = "truncated qhmat file";
        return 0;
    }
    uint8_t v = *r->p++;
    r->remaining--;
    r->hash = (r->hash ^ v) * FNV_PRIME;
    return v;
}

static uint32_t rd_u32(reader* r) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)rd_byte(r) << (8 * i);
    return v;
}

static uint64_t rd_u64(reader* r) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)rd_byte(r) << (8 * i);
    return v;
}

static double rd_f64(reader* r) {
    uint64_t b = rd_u64(r);
    double d;
    memcpy(&d, &b, 8);
    return d;
}

static int require_bytes(reader* r, uint64_t count, uint64_t width) {
    if (width != 0 && count > remaining_data(r) / width) {
        r->failed = 1;
        r->why = "truncated qhmat payload";
        return 0;
    }
    return 1;
}

static uint64_t words_for(uint64_t rows, int bits) { return (rows * (uint64_t)bits + 31) / 32; }

QHO_EXPORT void qho_free(qho_matrix* m) {
    if (!m) return;
    for (uint64_t b = 0; b < m->block_count; ++b) {
        qho_block* k = &m->blocks[b];
        free(k->values);
        free(k->widths);
        free(k->left_scales);
        free(k->right_scales);
        free(k->left_words);
        free(k->right_words);
        free(k->left_offsets);
        free(k->right_offsets);
    }
    free(m->blocks);
    free(m->permutation);
    free(m);
}

static int cmp_pair(const void* a, const void* b) {
    const uint64_t* x = (const uint64_t*)a;
    const uint64_t* y = (const uint64_t*)b;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    return 0;
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* finalize(): every elementary row slab's column intervals tile [0, order). */
static const char* check_cover(const qho_matrix* m) {
    if (m->block_count == 0) return "matrix has no blocks";
    uint64_t nb = 2 + 2 * m->block_count;
    uint64_t* bounds = (uint64_t*)malloc(nb * sizeof(uint64_t));
    uint64_t* iv = (uint64_t*)malloc(2 * m->block_count * sizeof(uint64_t));
    if (!bounds || !iv) {
        free(bounds);
        free(iv);
        return "out of memory";
    }
    bounds[0] = 0;
    bounds[1] = m->order;
    for (uint64_t b = 0; b < m->block_count; ++b) {
        bounds[2 + 2 * b] = m->blocks[b].row0;
        bounds[3 + 2 * b] = m->blocks[b].row1;
    }
    qsort(bounds, nb, sizeof(uint64_t), cmp_u64);
    uint64_t u = 0;
    for (uint64_t i = 0; i < nb; ++i)
        if (i == 0 || bounds[i] != bounds[u - 1]) bounds[u++] = bounds[i];
    const char* why = NULL;
    for (uint64_t s = 0; s + 1 < u && !why; ++s) {
        uint64_t cnt = 0;
        for (uint64_t b = 0; b < m->block_count; ++b) {
            const qho_block* k = &m->blocks[b];
            if (k->row0 <= bounds[s] && bounds[s] < k->row1) {
                iv[2 * cnt] = k->col0;
                iv[2 * cnt + 1] = k->col1;
                ++cnt;
            }
        }
        qsort(iv, cnt, 2 * sizeof(uint64_t), cmp_pair);
        uint64_t end = 0;
        for (uint64_t i = 0; i < cnt; ++i) {
            if (iv[2 * i] != end) {
                why = "block partition has a gap or overlap";
                break;
            }
            end = iv[2 * i + 1];
        }
        if (!why && end != m->order) why = "block partition does not cover the matrix";
    }
    free(bounds);
    free(iv);
    return why;
}

/* Parse a QHMAT001 byte image (io.cpp:173-257).  Returns NULL and fills err on
 * failure, with the reference's messages. */
QHO_EXPORT qho_matrix* qho_parse(const uint8_t* bytes, uint64_t len, char* err, size_t err_len) {
    reader r = {bytes, len, FNV_OFFSET, 0, NULL};
    qho_matrix* m = NULL;
    if (len < 24) {
        set_err(err, err_len, "truncated qhmat file");
        return NULL;
    }
    char magic[9] = {0};
    for (int i = 0; i < 8; ++i) magic[i] = (char)rd_byte(&r);
    if (r.failed) goto fail_reader;
    if (memcmp(magic, "QHMAT001", 8) != 0) {
        set_err(err, err_len, "invalid qhmat file magic");
        return NULL;
    }
    if (rd_u64(&r) != 1) {
        if (r.failed) goto fail_reader;
        set_err(err, err_len, "unsupported qhmat file version");
        return NULL;
    }
    uint64_t order = rd_u64(&r), count = rd_u64(&r);
    if (r.failed) goto fail_reader;
    if (!order || !count || order > remaining_data(&r) / 8) {
        set_err(err, err_len, "invalid qhmat file dimensions");
        return NULL;
    }
    m = (qho_matrix*)calloc(1, sizeof(qho_matrix));
    m->order = order;
    m->permutation = (uint64_t*)malloc(order * sizeof(uint64_t));
    for (uint64_t i = 0; i < order; ++i) m->permutation[i] = rd_u64(&r);
    if (r.failed) goto fail_reader;
    {
        /* HMatrix constructor: the permutation must be a bijection. */
        uint8_t* seen = (uint8_t*)calloc(order, 1);
        int ok = 1;
        for (uint64_t i = 0; i < order && ok; ++i) {
            uint64_t v = m->permutation[i];
            if (v >= order || seen[v]) ok = 0;
            else seen[v] = 1;
        }
        free(seen);
        if (!ok) {
            set_err(err, err_len, "permutation is not a bijection");
            goto fail;
        }
    }
    if (count > remaining_data(&r) / 34) {
        set_err(err, err_len, "invalid qhmat block count");
        goto fail;
    }
    m->blocks = (qho_block*)calloc(count, sizeof(qho_block));
    for (uint64_t k = 0; k < count; ++k) {
        qho_block* b = &m->blocks[k];
        m->block_count = k + 1; /* so qho_free releases what was read */
        b->row0 = rd_u64(&r);
        b->row1 = rd_u64(&r);
        b->col0 = rd_u64(&r);
        b->col1 = rd_u64(&r);
        uint8_t adm = rd_byte(&r), dense = rd_byte(&r);
        if (r.failed) goto fail_reader;
        if (adm > 1 || dense > 1) {
            set_err(err, err_len, "invalid qhmat block flag");
            goto fail;
        }
        b->admissible = adm;
        b->dense = dense;
        /* check_rectangle (core.cpp:214-222) */
        if (!(b->row0 < b->row1 && b->row1 <= order && b->col0 < b->col1 && b->col1 <= order)) {
            set_err(err, err_len, "invalid block rectangle");
            goto fail;
        }
        int same = b->row0 == b->col0 && b->row1 == b->col1;
        int disjoint = b->row1 <= b->col0 || b->col1 <= b->row0;
        if (dense ? !same : !disjoint) {
            set_err(err, err_len,
                    "only diagonal blocks may be dense; factorized blocks must be off-diagonal");
            goto fail;
        }
        uint64_t rows = b->row1 - b->row0, cols = b->col1 - b->col0;
        if (dense) {
            uint64_t total = rows * cols;
            if (!require_bytes(&r, total, 8)) goto fail_reader;
            b->values = (double*)malloc(total * sizeof(double));
            for (uint64_t i = 0; i < total; ++i) {
                b->values[i] = rd_f64(&r);
                if (!isfinite(b->values[i])) {
                    set_err(err, err_len, "nonfinite dense value");
                    goto fail;
                }
            }
        } else {
            uint64_t rank = rd_u64(&r);
            b->menu_size = rd_u64(&r);
            if (r.failed) goto fail_reader;
            uint64_t mn = rows < cols ? rows : cols;
            if (rank > mn || b->menu_size == 0 || b->menu_size > 31) {
                set_err(err, err_len, "invalid qhmat rank or precision menu");
                goto fail;
            }
            b->rank = rank;
            b->truncation_error = rd_f64(&r);
            b->quantization_bound = rd_f64(&r);
            if (r.failed) goto fail_reader;
            if (!isfinite(b->truncation_error) || b->truncation_error < 0 ||
                !isfinite(b->quantization_bound) || b->quantization_bound < 0) {
                set_err(err, err_len, "invalid qhmat error bound");
                goto fail;
            }
            if (!require_bytes(&r, rank, 17)) goto fail_reader;
            b->widths = (uint8_t*)malloc(rank ? rank : 1);
            for (uint64_t j = 0; j < rank; ++j) {
                b->widths[j] = rd_byte(&r);
                if (b->widths[j] < 2 || b->widths[j] > 32) {
                    set_err(err, err_len, "invalid qhmat bit width");
                    goto fail;
                }
            }
            b->left_scales = (double*)malloc((rank ? rank : 1) * sizeof(double));
            b->right_scales = (double*)malloc((rank ? rank : 1) * sizeof(double));
            for (uint64_t j = 0; j < rank; ++j) b->left_scales[j] = rd_f64(&r);
            for (uint64_t j = 0; j < rank; ++j) b->right_scales[j] = rd_f64(&r);
            if (r.failed) goto fail_reader;
            for (uint64_t j = 0; j < rank; ++j)
                if (!isfinite(b->left_scales[j]) || b->left_scales[j] < 0 ||
                    !isfinite(b->right_scales[j]) || b->right_scales[j] < 0) {
                    set_err(err, err_len, "invalid qhmat scale");
                    goto fail;
                }
            b->left_offsets = (uint64_t*)malloc((rank ? rank : 1) * sizeof(uint64_t));
            b->right_offsets = (uint64_t*)malloc((rank ? rank : 1) * sizeof(uint64_t));
            uint64_t lw = 0, rw = 0;
            for (uint64_t j = 0; j < rank; ++j) {
                b->left_offsets[j] = lw;
                b->right_offsets[j] = rw;
                lw += words_for(rows, b->widths[j]);
                rw += words_for(cols, b->widths[j]);
            }
            if (!require_bytes(&r, lw + rw, 4)) goto fail_reader;
            b->left_word_count = lw;
            b->right_word_count = rw;
            b->left_words = (uint32_t*)malloc((lw ? lw : 1) * sizeof(uint32_t));
            b->right_words = (uint32_t*)malloc((rw ? rw : 1) * sizeof(uint32_t));
            for (uint64_t i = 0; i < lw; ++i) b->left_words[i] = rd_u32(&r);
            for (uint64_t i = 0; i < rw; ++i) b->right_words[i] = rd_u32(&r);
            if (r.failed) goto fail_reader;
        }
    }
    /* Reader::finish (io.cpp:109-118) */
    if (r.remaining != 8) {
        set_err(err, err_len, "trailing qhmat data");
        goto fail;
    }
    {
        uint64_t checksum = 0;
        for (int i = 0; i < 8; ++i) checksum |= (uint64_t)r.p[i] << (8 * i);
        if (checksum != r.hash) {
            set_err(err, err_len, "qhmat checksum mismatch");
            goto fail;
        }
    }
    {
        const char* why = check_cover(m);
        if (why) {
            set_err(err, err_len, "%s", why);
            goto fail;
        }
    }
    return m;
fail_reader:
    set_err(err, err_len, "%s", r.why ? r.why : "truncated qhmat file");
fail:
    qho_free(m);
    return NULL;
}

/* ---------------------------------------------------------------- decode */

/* core.cpp:269-282: LSB-first bit field of `bits` at position row*bits within
 * the run that starts at word offsets[column]; sign-extended. */
static int64_t decode_code(const uint32_t* words, const uint64_t* offsets, uint64_t row,
                           uint64_t column, int bits) {
    uint64_t position = row * (uint64_t)bits;
    uint64_t word = offsets[column] + position / 32;
    unsigned shift = (unsigned)(position % 32);
    uint32_t raw = words[word] >> shift;
    if (shift + (unsigned)bits > 32) raw |= words[word + 1] << (32 - shift);
    uint32_t mask = bits == 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
    raw &= mask;
    return (raw & (1u << (bits - 1))) ? (int64_t)raw - ((int64_t)1 << bits) : (int64_t)raw;
}

static inline double decode_value(const uint32_t* words, const uint64_t* offsets,
                                  const double* scales, uint64_t row, uint64_t column,
                                  int bits) {
    return (double)decode_code(words, offsets, row, column, bits) * scales[column];
}

/* ------------------------------------------------------------- accessors */

QHO_EXPORT uint64_t qho_order(const qho_matrix* m) { return m->order; }
QHO_EXPORT uint64_t qho_block_count(const qho_matrix* m) { return m->block_count; }

/* info[0..9] = row0,row1,col0,col1,admissible,dense,rank,menu_size,
 * left_word_count,right_word_count */
QHO_EXPORT void qho_block_info(const qho_matrix* m, uint64_t b, uint64_t* info) {
    const qho_block* k = &m->blocks[b];
    info[0] = k->row0;
    info[1] = k->row1;
    info[2] = k->col0;
    info[3] = k->col1;
    info[4] = k->admissible;
    info[5] = k->dense;
    info[6] = k->rank;
    info[7] = k->menu_size;
    info[8] = k->left_word_count;
    info[9] = k->right_word_count;
}

QHO_EXPORT void qho_block_widths(const qho_matrix* m, uint64_t b, uint8_t* out) {
    memcpy(out, m->blocks[b].widths, m->blocks[b].rank);
}

/* All codes of one factor, component-major: out[j*rows + i] (side 0 = left/P,
 * side 1 = right/Q). */
QHO_EXPORT void qho_block_codes(const qho_matrix* m, uint64_t b, int side, int32_t* out) {
    const qho_block* k = &m->blocks[b];
    uint64_t rows = side == 0 ? k->row1 - k->row0 : k->col1 - k->col0;
    const uint32_t* w = side == 0 ? k->left_words : k->right_words;
    const uint64_t* off = side == 0 ? k->left_offsets : k->right_offsets;
    for (uint64_t j = 0; j < k->rank; ++j)
        for (uint64_t i = 0; i < rows; ++i)
            out[j * rows + i] = (int32_t)decode_code(w, off, i, j, k->widths[j]);
}

/* core.cpp:467-472 */
/* FNV-1a-64 of a byte range: the QHMAT001 trailer (io.cpp:18-19, 42).  Lets
 * the CPU baseline write images without loading the CUDA library. */
QHO_EXPORT uint64_t qho_fnv1a64(const uint8_t* bytes, uint64_t len) {
    uint64_t h = FNV_OFFSET;
    for (uint64_t i = 0; i < len; ++i) h = (h ^ bytes[i]) * FNV_PRIME;
    return h;
}

QHO_EXPORT double qho_bound(const qho_matrix* m) {
    double bound = 0.0;
    for (uint64_t b = 0; b < m->block_count; ++b) {
        double v = m->blocks[b].truncation_error + m->blocks[b].quantization_bound;
        if (v > bound) bound = v;
    }
    return bound;
}

/* ---------------------------------------------------------------- matmul */

typedef struct {
    const qho_matrix* m;
    const double* x;
    double* y;
    uint64_t rhs;
    uint64_t lo, hi; /* clustered rows owned */
} mm_task;

static void* matmul_range(void* arg) {
    mm_task* t = (mm_task*)arg;
    const qho_matrix* m = t->m;
    const uint64_t* perm = m->permutation;
    const uint64_t rhs = t->rhs;
    const double* x = t->x;
    double* y = t->y;
    for (uint64_t bi = 0; bi < m->block_count; ++bi) {
        const qho_block* b = &m->blocks[bi];
        if (b->row1 <= t->lo || b->row0 >= t->hi) continue;
        uint64_t n = b->col1 - b->col0;
        uint64_t i0 = (t->lo > b->row0 ? t->lo : b->row0) - b->row0;
        uint64_t i1 = (t->hi < b->row1 ? t->hi : b->row1) - b->row0;
        if (b->dense) {
            for (uint64_t i = i0; i < i1; ++i)
                for (uint64_t k = 0; k < n; ++k)
                    for (uint64_t p = 0; p < rhs; ++p)
                        y[perm[b->row0 + i] * rhs + p] +=
                            b->values[i * n + k] * x[perm[b->col0 + k] * rhs + p];
        } else {
            for (uint64_t p = 0; p < rhs; ++p)
                for (uint64_t j = 0; j < b->rank; ++j) {
                    double dot = 0.0;
                    for (uint64_t k = 0; k < n; ++k)
                        dot += decode_value(b->right_words, b->right_offsets, b->right_scales, k,
                                            j, b->widths[j]) *
                               x[perm[b->col0 + k] * rhs + p];
                    for (uint64_t i = i0; i < i1; ++i)
                        y[perm[b->row0 + i] * rhs + p] +=
                            decode_value(b->left_words, b->left_offsets, b->left_scales, i, j,
                                         b->widths[j]) *
                            dot;
                }
        }
    }
    return NULL;
}

/* y = A x for row-major order x rhs arrays in source index order
 * (core.cpp:360-390).  threads <= 1 runs the reference's loop as written. */
QHO_EXPORT int qho_matmul(const qho_matrix* m, const double* x, double* y, uint64_t rhs,
                          int threads, char* err, size_t err_len) {
    if (rhs == 0 || rhs > UINT64_MAX / m->order) {
        set_err(err, err_len, "right-hand-side shape mismatch");
        return 1;
    }
    uint64_t total = m->order * rhs;
    for (uint64_t i = 0; i < total; ++i)
        if (!isfinite(x[i])) {
            set_err(err, err_len, "nonfinite right-hand side");
            return 1;
        }
    memset(y, 0, total * sizeof(double));
    if (threads <= 1 || m->order < (uint64_t)threads) {
        mm_task t = {m, x, y, rhs, 0, m->order};
        matmul_range(&t);
        return 0;
    }
    pthread_t* tid = (pthread_t*)malloc(threads * sizeof(pthread_t));
    mm_task* tasks = (mm_task*)malloc(threads * sizeof(mm_task));
    for (int t = 0; t < threads; ++t) {
        tasks[t].m = m;
        tasks[t].x = x;
        tasks[t].y = y;
        tasks[t].rhs = rhs;
        tasks[t].lo = m->order * (uint64_t)t / (uint64_t)threads;
        tasks[t].hi = m->order * (uint64_t)(t + 1) / (uint64_t)threads;
        pthread_create(&tid[t], NULL, matmul_range, &tasks[t]);
    }
    for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
    free(tid);
    free(tasks);
    return 0;
}

/* core.cpp:392-410: dense n x n in source index order. */
QHO_EXPORT void qho_reconstruct(const qho_matrix* m, double* out) {
    const uint64_t n = m->order;
    const uint64_t* perm = m->permutation;
    memset(out, 0, n * n * sizeof(double));
    for (uint64_t bi = 0; bi < m->block_count; ++bi) {
        const qho_block* b = &m->blocks[bi];
        uint64_t rows = b->row1 - b->row0, cols = b->col1 - b->col0;
        for (uint64_t i = 0; i < rows; ++i)
            for (uint64_t k = 0; k < cols; ++k) {
                double v = b->dense ? b->values[i * cols + k] : 0.0;
                for (uint64_t j = 0; j < b->rank; ++j)
                    v += decode_value(b->left_words, b->left_offsets, b->left_scales, i, j,
                                      b->widths[j]) *
                         decode_value(b->right_words, b->right_offsets, b->right_scales, k, j,
                                      b->widths[j]);
                out[perm[b->row0 + i] * n + perm[b->col0 + k]] = v;
            }
    }
}

/* ------------------------------------------------------------------ pack */

/* core.cpp:235-267.  matrix is column-major rows x ncomp (matrix[j*rows+i]).
 * words must hold sum_j ceil(rows*widths[j]/32) zeroed words; offsets and
 * scales receive ncomp entries. */
QHO_EXPORT void qho_pack(const double* matrix, uint64_t rows, const int* widths, uint64_t ncomp,
                         uint32_t* words, uint64_t* offsets, double* scales) {
    uint64_t used = 0;
    for (uint64_t j = 0; j < ncomp; ++j) {
        const int bits = widths[j];
        const uint64_t q = ((uint64_t)1 << (bits - 1)) - 1;
        double maximum = 0.0;
        for (uint64_t i = 0; i < rows; ++i) {
            double a = fabs(matrix[j * rows + i]);
            if (a > maximum) maximum = a;
        }
        const double scale = maximum == 0 ? 0 : maximum / (double)q;
        scales[j] = scale;
        offsets[j] = used;
        const uint64_t word_count = (rows * (uint64_t)bits + 31) / 32;
        memset(words + used, 0, word_count * sizeof(uint32_t));
        used += word_count;
        for (uint64_t i = 0; i < rows; ++i) {
            const double scaled = scale == 0 ? 0 : matrix[j * rows + i] / scale;
            int64_t rounded = (int64_t)nearbyint(scaled);
            int64_t lim = (int64_t)q;
            int64_t clipped = rounded < -lim ? -lim : (rounded > lim ? lim : rounded);
            const uint32_t mask = bits == 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
            const uint32_t raw = (uint32_t)clipped & mask;
            const uint64_t position = i * (uint64_t)bits;
            const uint64_t word = offsets[j] + position / 32;
            const unsigned shift = (unsigned)(position % 32);
            words[word] |= raw << shift;
            if (shift + (unsigned)bits > 32) words[word + 1] |= raw >> (32 - shift);
        }
    }
}
