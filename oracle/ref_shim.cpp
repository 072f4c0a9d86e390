// Test infrastructure only: a C-ABI shim over the reference's own C++ core
// (src/qhmat/core.cpp, src/qhmat/io.cpp), compiled straight from the
// reference's sources by oracle/build_ref.py into oracle/_ref/.  Nothing in the
// product links or loads this; tests and the bench's CPU-baseline leg use it to
// pin the plain-C restatement in oracle/qhmat_oracle.c and to time the
// reference's single-threaded HMatrix::matmul.
//
// Every entry point calls a public member of qhmat::HMatrix (core.hpp:52-75):
//   qhref_load        -> HMatrix::load            (io.cpp:173-257)
//   qhref_matmul      -> HMatrix::matmul          (core.cpp:360-390)
//   qhref_reconstruct -> HMatrix::reconstruct     (core.cpp:392-410)
//   qhref_bound       -> HMatrix::reconstruction_bound (core.cpp:467-472)
#include "qhmat/core.hpp"

#include <cstdio>
#include <cstring>
#include <exception>
#include <new>
#include <vector>

namespace {
void put_error(char* err, std::size_t len, const char* what) {
    if (err && len) {
        std::snprintf(err, len, "%s", what);
    }
}
}  // namespace

extern "C" {

void* qhref_load(const char* path, char* err, std::size_t err_len) {
    try {
        return new qhmat::HMatrix(qhmat::HMatrix::load(path));
    } catch (const std::exception& e) {
        put_error(err, err_len, e.what());
        return nullptr;
    }
}

void qhref_free(void* handle) { delete static_cast<qhmat::HMatrix*>(handle); }

std::size_t qhref_order(const void* handle) {
    return static_cast<const qhmat::HMatrix*>(handle)->order();
}

double qhref_bound(const void* handle) {
    return static_cast<const qhmat::HMatrix*>(handle)->reconstruction_bound();
}

// x and y are row-major order x rhs in source index order, as the reference's
// matmul takes them.
int qhref_matmul(const void* handle, const double* x, double* y, std::size_t rhs,
                 char* err, std::size_t err_len) {
    try {
        const auto* m = static_cast<const qhmat::HMatrix*>(handle);
        std::vector<double> xv(x, x + m->order() * rhs);
        std::vector<double> yv = m->matmul(xv, rhs);
        std::memcpy(y, yv.data(), yv.size() * sizeof(double));
        return 0;
    } catch (const std::exception& e) {
        put_error(err, err_len, e.what());
        return 1;
    }
}

int qhref_reconstruct(const void* handle, double* out, char* err, std::size_t err_len) {
    try {
        const auto* m = static_cast<const qhmat::HMatrix*>(handle);
        std::vector<double> d = m->reconstruct();
        std::memcpy(out, d.data(), d.size() * sizeof(double));
        return 0;
    } catch (const std::exception& e) {
        put_error(err, err_len, e.what());
        return 1;
    }
}

}  // extern "C"
