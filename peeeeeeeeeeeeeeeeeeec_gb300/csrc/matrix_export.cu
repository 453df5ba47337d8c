// Matrix Market export of the PEEC matrices (drop-in for the reference's
// include/matrix_export.h; host code).
//
// Reference (paths inside the reference project):
//   src/io/matrix_export.c:11-103    the directory (parents too, 0755) and
//                                    the file paths inside it
//   src/io/matrix_export.c:105-176   dense "array real general", values column
//                                    by column, one "%.17e" per line
//   src/io/matrix_export.c:178-258   incidence as 2 Ne 1-based coordinates
//   src/io/matrix_export.c:260-321   diagonal resistance as coordinates
//   src/io/matrix_export.c:323-432   L, A, P, PAT, R into one directory
//
// The file format (header lines and value formatting) is kept identical, so
// the files are byte-identical to the reference's.  The dense writer is the
// slow part (25 bytes of decimal text per value, 31 M values for the 5 cm
// box's Lp): columns are formatted in parallel host threads, a block of
// columns at a time, and the blocks are written in order.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <filesystem>
#include <string>
#include <thread>
#include <vector>

#include "../../include/matrix_export.h"

namespace {

namespace fs = std::filesystem;

// The directory and its missing parents (permissions 0755 as the
// reference's exporter creates them); an existing directory is fine.
int ensure_directory(const char *directory) {
    if (!directory || directory[0] == '\0') return -1;
    std::error_code ec;
    const fs::path dir(directory);
    if (fs::is_directory(dir, ec)) return 0;
    fs::create_directories(dir, ec);
    if (ec) {
        fprintf(stderr, "ERROR: cannot create directory '%s': %s\n", directory, ec.message().c_str());
        return -1;
    }
    fs::permissions(dir, fs::perms::owner_all | fs::perms::group_read | fs::perms::group_exec |
                             fs::perms::others_read | fs::perms::others_exec, ec);
    return 0;
}

// directory / file, or an empty string when a path argument is missing.
std::string join_path(const char *directory, const char *file) {
    if (!directory || !file) return std::string();
    return (fs::path(directory) / file).string();
}

// "%.17e\n" of data[row * cols + col] for rows 0.. of columns [c0, c1),
// column after column, appended to out
void format_columns(const double *data, size_t rows, size_t cols, size_t c0, size_t c1, std::string &out) {
    char line[40];
    out.clear();
    out.reserve((c1 - c0) * rows * 25);
    for (size_t col = c0; col < c1; ++col)
        for (size_t row = 0; row < rows; ++row) {
            const int k = snprintf(line, sizeof(line), "%.17e\n", data[row * cols + col]);
            out.append(line, (size_t)k);
        }
}

}  // namespace

extern "C" {

int matrix_export_dense_mtx(const char *filename, const double *data, size_t rows, size_t cols) {
    if (!filename || !data || rows == 0 || cols == 0) return -1;
    FILE *file = fopen(filename, "w");
    if (!file) {
        fprintf(stderr, "ERROR: cannot open matrix file '%s'.\n", filename);
        return -1;
    }
    fprintf(file, "%%%%MatrixMarket matrix array real general\n");
    fprintf(file, "%% PEEC matrix export\n");
    fprintf(file, "%zu %zu\n", rows, cols);
    unsigned hw = std::thread::hardware_concurrency();
    const size_t threads = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, 64));
    // blocks of about 4 M values, split over the threads by columns
    const size_t per_block = std::max<size_t>(threads, (4u << 20) / rows + 1);
    std::vector<std::string> parts(threads);
    bool ok = true;
    for (size_t b0 = 0; b0 < cols && ok; b0 += per_block) {
        const size_t b1 = std::min(cols, b0 + per_block), span = b1 - b0;
        std::vector<std::thread> pool;
        for (size_t t = 0; t < threads; ++t) {
            const size_t c0 = b0 + span * t / threads, c1 = b0 + span * (t + 1) / threads;
            if (c0 == c1) {
                parts[t].clear();
                continue;
            }
            pool.emplace_back(format_columns, data, rows, cols, c0, c1, std::ref(parts[t]));
        }
        for (auto &th : pool) th.join();
        for (const auto &p : parts)
            if (!p.empty() && fwrite(p.data(), 1, p.size(), file) != p.size()) ok = false;
    }
    if (fclose(file) != 0) ok = false;
    return ok ? 0 : -1;
}

int matrix_export_incidence_mtx(const char *filename, const Mesh *mesh) {
    if (!filename || !mesh || !mesh->edges || mesh->n_edges == 0 || mesh->n_nodes == 0) return -1;
    FILE *file = fopen(filename, "w");
    if (!file) return -1;
    fprintf(file, "%%%%MatrixMarket matrix coordinate real general\n");
    fprintf(file, "%% Incidence matrix A: Ne x Nv\n");
    fprintf(file, "%zu %zu %zu\n", mesh->n_edges, mesh->n_nodes, 2 * mesh->n_edges);
    for (size_t e = 0; e < mesh->n_edges; ++e) {
        fprintf(file, "%zu %d -1.0\n", e + 1, mesh->edges[2 * e] + 1);
        fprintf(file, "%zu %d 1.0\n", e + 1, mesh->edges[2 * e + 1] + 1);
    }
    fclose(file);
    return 0;
}

int matrix_export_resistance_mtx(const char *filename, const ResistanceMatrix *R) {
    if (!filename || !R || !R->diagonal || R->n == 0) return -1;
    FILE *file = fopen(filename, "w");
    if (!file) return -1;
    fprintf(file, "%%%%MatrixMarket matrix coordinate real general\n");
    fprintf(file, "%% Diagonal PEEC resistance matrix R\n");
    fprintf(file, "%zu %zu %zu\n", R->n, R->n, R->n);
    for (size_t i = 0; i < R->n; ++i) fprintf(file, "%zu %zu %.17e\n", i + 1, i + 1, R->diagonal[i]);
    fclose(file);
    return 0;
}

int matrix_export_peec_set(const char *directory, const Mesh *mesh, const InductanceMatrix *L,
                           const PotentialMatrix *P, const Matrix *PAT, const ResistanceMatrix *R) {
    if (!directory || !mesh || !L || !P || !PAT || !R) return -1;
    if (ensure_directory(directory) != 0) return -1;
    const std::string l = join_path(directory, "L.mtx"), a = join_path(directory, "A.mtx"),
                      p = join_path(directory, "P.mtx"), pat = join_path(directory, "PAT.mtx"),
                      r = join_path(directory, "R.mtx");
    if (matrix_export_dense_mtx(l.c_str(), L->data, L->n, L->n) || matrix_export_incidence_mtx(a.c_str(), mesh) ||
        matrix_export_dense_mtx(p.c_str(), P->data, P->n, P->n) ||
        matrix_export_dense_mtx(pat.c_str(), PAT->data, PAT->rows, PAT->cols) ||
        matrix_export_resistance_mtx(r.c_str(), R))
        return -1;
    printf("PEEC matrices saved : %s\n", directory);
    return 0;
}

}  // extern "C"
