// Seeded synthetic CSR inputs for the benchmark workloads (host code,
// libspg_synth.so).  Every row draws from its own counter-based stream
// (SplitMix64 of seed and row), so the matrices do not depend on the number of
// OpenMP threads.  Columns of every generated row are distinct and sorted;
// values are U[-1, 1) unless stated otherwise.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" {
typedef struct {
    int32_t rows, cols;
    int64_t nnz;
    int64_t* row_ptr;
    int32_t* col;
    double* val;
} spg_synth_csr;
}

namespace {

inline uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s;
    Rng(uint64_t seed, uint64_t stream) : s(seed * 0x9E3779B97F4A7C15ull ^ (stream + 0x632BE59BD9B4E019ull)) {
        splitmix(s);
    }
    uint64_t next() { return splitmix(s); }
    double unit() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }  // [0, 1)
    int64_t below(int64_t n) { return static_cast<int64_t>((static_cast<unsigned __int128>(next()) * static_cast<uint64_t>(n)) >> 64); }
    double sym() { return 2.0 * unit() - 1.0; }  // [-1, 1)
    double normal() {  // Box-Muller
        double u1 = unit();
        while (u1 <= 0.0) u1 = unit();
        const double u2 = unit();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

bool export_rows(int32_t rows, int32_t cols, const std::vector<std::vector<int32_t>>& rc,
                 const std::vector<std::vector<double>>& rv, spg_synth_csr* out) {
    out->rows = rows;
    out->cols = cols;
    out->row_ptr = static_cast<int64_t*>(std::malloc(sizeof(int64_t) * (static_cast<size_t>(rows) + 1)));
    if (!out->row_ptr) return false;
    out->row_ptr[0] = 0;
    for (int32_t r = 0; r < rows; ++r) out->row_ptr[r + 1] = out->row_ptr[r] + static_cast<int64_t>(rc[r].size());
    out->nnz = out->row_ptr[rows];
    out->col = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * std::max<int64_t>(1, out->nnz)));
    out->val = static_cast<double*>(std::malloc(sizeof(double) * std::max<int64_t>(1, out->nnz)));
    if (!out->col || !out->val) return false;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t r = 0; r < rows; ++r) {
        std::memcpy(out->col + out->row_ptr[r], rc[r].data(), sizeof(int32_t) * rc[r].size());
        std::memcpy(out->val + out->row_ptr[r], rv[r].data(), sizeof(double) * rv[r].size());
    }
    return true;
}

// k distinct values in [lo, hi] (k <= hi - lo + 1), Floyd's sampling, sorted.
void distinct_sorted(Rng& g, int64_t lo, int64_t hi, int64_t k, std::vector<int32_t>& out) {
    out.clear();
    const int64_t n = hi - lo + 1;
    if (k >= n) {
        for (int64_t c = lo; c <= hi; ++c) out.push_back(static_cast<int32_t>(c));
        return;
    }
    std::vector<int64_t> pick;
    pick.reserve(static_cast<size_t>(k));
    for (int64_t j = n - k; j < n; ++j) {
        const int64_t t = g.below(j + 1);
        if (std::find(pick.begin(), pick.end(), t) == pick.end()) pick.push_back(t);
        else pick.push_back(j);
    }
    for (int64_t p : pick) out.push_back(static_cast<int32_t>(lo + p));
    std::sort(out.begin(), out.end());
}

}  // namespace

extern "C" {

void spg_synth_free(spg_synth_csr* m) {
    if (!m) return;
    std::free(m->row_ptr);
    std::free(m->col);
    std::free(m->val);
    m->row_ptr = nullptr;
    m->col = nullptr;
    m->val = nullptr;
}

// rows x cols, per row a length drawn uniformly from [min_len, max_len] (equal
// bounds: a fixed length) of distinct uniform columns; values U[-1, 1).
int spg_synth_uniform(int32_t rows, int32_t cols, int32_t min_len, int32_t max_len, uint64_t seed,
                      spg_synth_csr* out) {
    if (rows < 0 || cols <= 0 || min_len < 0 || max_len < min_len || max_len > cols) return 1;
    std::vector<std::vector<int32_t>> rc(static_cast<size_t>(rows));
    std::vector<std::vector<double>> rv(static_cast<size_t>(rows));
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t r = 0; r < rows; ++r) {
        Rng g(seed, static_cast<uint64_t>(r));
        const int64_t len = min_len + (max_len > min_len ? g.below(max_len - min_len + 1) : 0);
        distinct_sorted(g, 0, cols - 1, len, rc[r]);
        rv[r].resize(rc[r].size());
        for (auto& v : rv[r]) v = g.sym();
    }
    return export_rows(rows, cols, rc, rv, out) ? 0 : 2;
}

// n x n with lognormal row lengths: len = round(exp(mu + sigma*N(0,1))),
// mu = ln(mean) - sigma^2/2 (arithmetic mean `mean`), clamped to [1, max_len].
// Each entry lies with probability band_frac in [i - band, i + band] (clipped
// to the matrix) and otherwise anywhere in [0, n); columns are distinct (a
// saturated band spills into the uniform part).  Values U[-1, 1).
int spg_synth_powerlaw(int32_t n, double mean, double sigma, int32_t max_len, int32_t band, double band_frac,
                       uint64_t seed, spg_synth_csr* out) {
    if (n <= 0 || mean <= 0 || sigma < 0 || max_len < 1 || band < 0) return 1;
    const double mu = std::log(mean) - 0.5 * sigma * sigma;
    std::vector<std::vector<int32_t>> rc(static_cast<size_t>(n));
    std::vector<std::vector<double>> rv(static_cast<size_t>(n));
#pragma omp parallel for schedule(dynamic, 256)
    for (int32_t r = 0; r < n; ++r) {
        Rng g(seed, static_cast<uint64_t>(r));
        int64_t len = std::llround(std::exp(mu + sigma * g.normal()));
        len = std::min<int64_t>(std::max<int64_t>(len, 1), std::min<int64_t>(max_len, n));
        const int64_t lo = std::max<int64_t>(0, static_cast<int64_t>(r) - band);
        const int64_t hi = std::min<int64_t>(n - 1, static_cast<int64_t>(r) + band);
        const int64_t band_cap = hi - lo + 1;
        int64_t in_band = 0;
        for (int64_t e = 0; e < len; ++e) in_band += g.unit() < band_frac;
        in_band = std::min(in_band, band_cap);
        std::vector<int32_t> a, b;
        distinct_sorted(g, lo, hi, in_band, a);
        // uniform part: distinct, and distinct from the band part
        std::vector<int32_t>& cols = rc[r];
        cols = a;
        const int64_t want = len;
        while (static_cast<int64_t>(cols.size()) < want) {
            const int32_t c = static_cast<int32_t>(g.below(n));
            if (!std::binary_search(a.begin(), a.end(), c) && std::find(b.begin(), b.end(), c) == b.end()) {
                b.push_back(c);
                cols.push_back(c);
            }
        }
        std::sort(cols.begin(), cols.end());
        rv[r].resize(cols.size());
        for (auto& v : rv[r]) v = g.sym();
    }
    return export_rows(n, n, rc, rv, out) ? 0 : 2;
}

// 7-point Laplacian on an nx*ny*nz grid (row = x + nx*(y + ny*z)): 6 on the
// diagonal, -1 for each existing neighbour, columns sorted.
int spg_synth_laplacian3d(int32_t nx, int32_t ny, int32_t nz, spg_synth_csr* out) {
    const int64_t n = static_cast<int64_t>(nx) * ny * nz;
    if (nx <= 0 || ny <= 0 || nz <= 0 || n > INT32_MAX) return 1;
    std::vector<std::vector<int32_t>> rc(static_cast<size_t>(n));
    std::vector<std::vector<double>> rv(static_cast<size_t>(n));
#pragma omp parallel for schedule(static, 4096)
    for (int64_t r = 0; r < n; ++r) {
        const int64_t x = r % nx, y = (r / nx) % ny, z = r / (static_cast<int64_t>(nx) * ny);
        auto& c = rc[r];
        auto& v = rv[r];
        auto add = [&](int64_t col, double val) {
            c.push_back(static_cast<int32_t>(col));
            v.push_back(val);
        };
        const int64_t sxy = static_cast<int64_t>(nx) * ny;
        if (z > 0) add(r - sxy, -1.0);
        if (y > 0) add(r - nx, -1.0);
        if (x > 0) add(r - 1, -1.0);
        add(r, 6.0);
        if (x + 1 < nx) add(r + 1, -1.0);
        if (y + 1 < ny) add(r + nx, -1.0);
        if (z + 1 < nz) add(r + sxy, -1.0);
    }
    return export_rows(static_cast<int32_t>(n), static_cast<int32_t>(n), rc, rv, out) ? 0 : 2;
}

// Restriction R aggregating 2x2x2 blocks of an nx*ny*nz grid (even sizes):
// coarse row c = X + (nx/2)*(Y + (ny/2)*Z) has value 1/8 at the 8 fine points
// of its block.  transpose != 0 returns R^T (fine rows, one entry each).
int spg_synth_restriction(int32_t nx, int32_t ny, int32_t nz, int32_t transpose, spg_synth_csr* out) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx % 2 || ny % 2 || nz % 2) return 1;
    const int64_t n = static_cast<int64_t>(nx) * ny * nz;
    const int64_t cx = nx / 2, cy = ny / 2, cz = nz / 2, nc = cx * cy * cz;
    if (n > INT32_MAX) return 1;
    if (!transpose) {
        std::vector<std::vector<int32_t>> rc(static_cast<size_t>(nc));
        std::vector<std::vector<double>> rv(static_cast<size_t>(nc));
#pragma omp parallel for schedule(static, 4096)
        for (int64_t c = 0; c < nc; ++c) {
            const int64_t X = c % cx, Y = (c / cx) % cy, Z = c / (cx * cy);
            for (int dz = 0; dz < 2; ++dz)
                for (int dy = 0; dy < 2; ++dy)
                    for (int dx = 0; dx < 2; ++dx) {
                        const int64_t f = (2 * X + dx) + nx * ((2 * Y + dy) + static_cast<int64_t>(ny) * (2 * Z + dz));
                        rc[c].push_back(static_cast<int32_t>(f));
                    }
            std::sort(rc[c].begin(), rc[c].end());
            rv[c].assign(rc[c].size(), 0.125);
        }
        return export_rows(static_cast<int32_t>(nc), static_cast<int32_t>(n), rc, rv, out) ? 0 : 2;
    }
    std::vector<std::vector<int32_t>> rc(static_cast<size_t>(n));
    std::vector<std::vector<double>> rv(static_cast<size_t>(n));
#pragma omp parallel for schedule(static, 4096)
    for (int64_t f = 0; f < n; ++f) {
        const int64_t x = f % nx, y = (f / nx) % ny, z = f / (static_cast<int64_t>(nx) * ny);
        rc[f].push_back(static_cast<int32_t>((x / 2) + cx * ((y / 2) + cy * (z / 2))));
        rv[f].push_back(0.125);
    }
    return export_rows(static_cast<int32_t>(n), static_cast<int32_t>(nc), rc, rv, out) ? 0 : 2;
}

}  // extern "C"
