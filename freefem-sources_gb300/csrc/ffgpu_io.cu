// ffgpu_io.cu -- FreeFEM's sparse-matrix text forms (host code, no device).
//
// FreeFEM prints a matrix (`ofstream f("A.txt"); f << A;`, and the `.matrix` file of
// `solve(..., save="name")`) with HashMatrix's operator<< (HashMatrix.hpp:484-520):
//   "#  HashMatrix Matrix (COO) <address>" / "#    n  m  nnz  half  fortran  state" header,
//     then "n m nnz half fortran state type_state" and one "i j a_ij" line per entry, indices
//     from `fortran` (0 or 1), values at 20 significant digits;
//   "# Sparse Matrix (Morse) <address>" when the matrix is held as CSR: "n m half nnz", then
//     1-based "i j a_ij" in row order, values below 1e-305 printed as 0.
// It reads both back (HashMatrix(istream&), HashMatrix.cpp:137-214, with WhichMatrix's test on
// the first comment line), every entry assigned -- a repeated (i, j) keeps its last value.
#include "ffgpu_internal.cuh"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace ffgpu {
namespace {

struct Triple {
    int64_t seq;
    int32_t i, j;
    double a;
};

// reads the whole file; kind 2 = Morse, 3 = COO (WhichMatrix)
int parse_matrix_text(const char *path, int &n, int &m, int &half, std::vector<Triple> &t) {
    FILE *f = fopen(path, "r");
    if (!f) { set_error("cannot open %s", path); return FFGPU_EINVAL; }
    int c;
    while ((c = fgetc(f)) != EOF && isspace(c)) {}
    int kind = 0;
    // comment lines; the first one names the form
    bool first_line = true;
    while (c == '#') {
        std::string line;
        while ((c = fgetc(f)) != EOF && c != '\n' && c != '\r') line += (char)c;
        if (first_line) {
            if (line.find("(Morse)") != std::string::npos) kind = 2;
            else if (line.find("(COO)") != std::string::npos) kind = 3;
            first_line = false;
        }
        while (c != EOF && isspace(c)) c = fgetc(f);
    }
    if (c != EOF) ungetc(c, f);
    int rc = FFGPU_OK;
    long long nnz = 0;
    int fortran = 1;
    if (kind == 2) {
        if (fscanf(f, "%d %d %d %lld", &n, &m, &half, &nnz) != 4) rc = FFGPU_EINVAL;
    } else if (kind == 3) {
        int st = 0, ts = 0;
        if (fscanf(f, "%d %d %lld %d %d %d %d", &n, &m, &nnz, &half, &fortran, &st, &ts) != 7) rc = FFGPU_EINVAL;
    } else {
        fclose(f);
        set_error("%s: not a FreeFEM matrix (no '(Morse)' or '(COO)' header)", path);
        return FFGPU_EINVAL;
    }
    if (!rc && (n < 0 || m < 0 || nnz < 0 || n > INT32_MAX - 1 || nnz > INT32_MAX)) rc = FFGPU_EINVAL;
    if (rc) { fclose(f); set_error("%s: bad size line", path); return rc; }
    t.clear();
    t.reserve((size_t)nnz);
    for (long long k = 0; k < nnz; ++k) {
        long long ii, jj;
        double a;
        if (fscanf(f, "%lld %lld %lf", &ii, &jj, &a) != 3) {
            fclose(f);
            set_error("%s: entry %lld of %lld unreadable", path, k, nnz);
            return FFGPU_EINVAL;
        }
        ii -= fortran;
        jj -= fortran;
        if (ii < 0 || ii >= n || jj < 0 || jj >= m) {
            fclose(f);
            set_error("%s: entry %lld (%lld, %lld) outside the %d x %d matrix", path, k, ii, jj, n, m);
            return FFGPU_EINVAL;
        }
        t.push_back(Triple{(int64_t)k, (int32_t)ii, (int32_t)jj, a});
    }
    fclose(f);
    // row-major order; a repeated (i, j) keeps its last value (entries are assigned)
    std::stable_sort(t.begin(), t.end(), [](const Triple &x, const Triple &y) {
        return x.i != y.i ? x.i < y.i : x.j < y.j;
    });
    size_t w = 0;
    for (size_t k = 0; k < t.size(); ++k) {
        if (w > 0 && t[w - 1].i == t[k].i && t[w - 1].j == t[k].j) t[w - 1] = t[k];
        else t[w++] = t[k];
    }
    t.resize(w);
    return FFGPU_OK;
}

}  // namespace
}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_matrix_text_read(const char *path, int *n, int *m, int64_t *nnz, int *half, int32_t *rowptr,
                           int32_t *col, double *val) {
    FFGPU_CHECK(path && n && m && nnz && half, FFGPU_EINVAL, "ffgpu_matrix_text_read: NULL argument");
    std::vector<Triple> t;
    int nn = 0, mm = 0, hh = 0;
    try {
        FFGPU_TRY(parse_matrix_text(path, nn, mm, hh, t));
    } catch (const std::bad_alloc &) {
        set_error("%s: out of host memory", path);
        return FFGPU_ENOMEM;
    }
    *n = nn; *m = mm; *half = hh;
    *nnz = (int64_t)t.size();
    if (!rowptr) return FFGPU_OK;
    FFGPU_CHECK(col && val, FFGPU_EINVAL, "ffgpu_matrix_text_read: NULL col/val");
    for (int i = 0; i <= nn; ++i) rowptr[i] = 0;
    for (size_t k = 0; k < t.size(); ++k) {
        rowptr[t[k].i + 1]++;
        col[k] = t[k].j;
        val[k] = t[k].a;
    }
    for (int i = 0; i < nn; ++i) rowptr[i + 1] += rowptr[i];
    return FFGPU_OK;
}

int ffgpu_matrix_text_write(const char *path, int format, int n, int m, int half, const int32_t *rowptr,
                            const int32_t *col, const double *val) {
    FFGPU_CHECK(path && rowptr && (rowptr[n] == 0 || (col && val)) && n >= 0 && m >= 0, FFGPU_EINVAL,
                "ffgpu_matrix_text_write: bad argument");
    FFGPU_CHECK(format == FFGPU_TEXT_COO || format == FFGPU_TEXT_MORSE, FFGPU_EINVAL,
                "ffgpu_matrix_text_write: unknown format %d", format);
    FILE *f = fopen(path, "w");
    if (!f) { set_error("cannot write %s", path); return FFGPU_EINVAL; }
    const long long nnz = rowptr[n];
    if (format == FFGPU_TEXT_MORSE) {
        fprintf(f, "# Sparse Matrix (Morse)  %p\n", (const void *)rowptr);
        fprintf(f, "# first line: n m (is symmetic) nnz \n");
        fprintf(f, "# after for each nonzero coefficient:   i j a_ij where (i,j) \\in  {1,...,n}x{1,...,m} \n");
        fprintf(f, "%d %d %d  %lld\n", n, m, half, nnz);
        for (int i = 0; i < n; ++i)
            for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                const double a = std::fabs(val[k]) < 1e-305 ? 0.0 : val[k];
                fprintf(f, "%9d %9d %.20g\n", i + 1, col[k] + 1, a);
            }
    } else {
        // sorted (state 2) CSR-ordered COO, 0-based: what FreeFEM prints once [I,J,C]=A sorted it
        fprintf(f, "#  HashMatrix Matrix (COO) %p\n", (const void *)rowptr);
        fprintf(f, "#    n       m        nnz     half     fortran   state  \n");
        fprintf(f, "%d %d %lld %d 0 2 1 \n", n, m, nnz, half);
        for (int i = 0; i < n; ++i)
            for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) fprintf(f, "%10d%10d %.20g\n", i, col[k], val[k]);
    }
    const bool ok = !ferror(f);
    fclose(f);
    if (!ok) { set_error("write error on %s", path); return FFGPU_EINVAL; }
    return FFGPU_OK;
}

}  // extern "C"
