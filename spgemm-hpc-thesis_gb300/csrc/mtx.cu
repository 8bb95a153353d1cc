// Matrix Market reader with the semantics of the reference's readMatrixMarket
// (src/common/matrix_market.cpp:28-145): coordinate matrices with real,
// integer or pattern fields, general / symmetric / skew-symmetric / hermitian
// storage (mirrored entries appended right after their entry, negated for
// skew-symmetric), comment and empty lines skipped anywhere, Fortran 'D'
// exponents accepted, every entry kept in file order (duplicates included),
// rows assembled by a stable counting sort.  Entry lines are parsed with the
// same stream extraction the reference uses, so the same inputs are accepted
// and rejected.  The entry lines are split into one chunk per host thread and
// parsed in parallel; the first error in file order is the one reported.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/spgemm_gb300.h"

namespace {

struct Entry {
    int32_t row, column;
    double value;
};

struct FormatError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

std::string lower(std::string s) {
    for (char& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    return s;
}

bool blank_or_comment(const char* b, const char* e) {
    while (b < e && (*b == ' ' || *b == '\t' || *b == '\r' || *b == '\n')) ++b;
    return b == e || *b == '%';
}

enum Sym { kGeneral, kSymmetric, kSkew, kHermitian };

struct Header {
    bool pattern = false;
    Sym sym = kGeneral;
    int rows = 0, cols = 0;
    int64_t entries = 0;
};

struct Chunk {
    std::vector<Entry> out;
    int64_t data_lines = 0;     // entry lines seen in the chunk
    int64_t error_line = -1;    // index (among the chunk's entry lines) of the first bad line
    std::string error;
};

// One entry line (a copy: 'D'/'d' exponents become 'E'/'e' first).
bool parse_entry(std::string line, const Header& h, Entry& e, std::string& why) {
    std::replace(line.begin(), line.end(), 'D', 'E');
    std::replace(line.begin(), line.end(), 'd', 'e');
    std::istringstream in(line);
    int row = 0, column = 0;
    double value = 1.0;
    std::string extra;
    if (!(in >> row >> column) || (!h.pattern && !(in >> value)) || !std::isfinite(value) || (in >> extra)) {
        why = "invalid Matrix Market entry";
        return false;
    }
    if (row < 1 || row > h.rows || column < 1 || column > h.cols) {
        why = "Matrix Market entry index is out of range";
        return false;
    }
    e.row = row - 1;
    e.column = column - 1;
    e.value = value;
    if (h.sym == kSkew && e.row == e.column && value != 0.0) {
        why = "skew-symmetric diagonal must be zero";
        return false;
    }
    return true;
}

void parse_chunk(const char* b, const char* e, const Header& h, Chunk& c) {
    const bool mirrored = h.sym != kGeneral;
    while (b < e) {
        const char* nl = static_cast<const char*>(std::memchr(b, '\n', static_cast<size_t>(e - b)));
        const char* end = nl ? nl : e;
        if (!blank_or_comment(b, end)) {
            Entry en;
            std::string why;
            if (c.error_line < 0 && !parse_entry(std::string(b, end), h, en, why)) {
                c.error_line = c.data_lines;
                c.error = why;
            }
            if (c.error_line < 0) {
                c.out.push_back(en);
                if (mirrored && en.row != en.column)
                    c.out.push_back({en.column, en.row, h.sym == kSkew ? -en.value : en.value});
            }
            ++c.data_lines;
        }
        b = nl ? nl + 1 : e;
    }
}

void read_all(const char* path, std::vector<char>& buf) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw FormatError(std::string("cannot open Matrix Market file: ") + path);
    in.seekg(0, std::ios::end);
    const std::streamoff n = in.tellg();
    in.seekg(0, std::ios::beg);
    buf.resize(static_cast<size_t>(n > 0 ? n : 0));
    if (n > 0) in.read(buf.data(), n);
}

void parse_file(const char* path, int32_t& rows, int32_t& cols, std::vector<int64_t>& rp, std::vector<int32_t>& ci,
                std::vector<double>& va) {
    std::vector<char> buf;
    read_all(path, buf);
    const char* p = buf.data();
    const char* end = p + buf.size();
    auto next_line = [&](std::string& line) -> bool {
        if (p >= end) return false;
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', static_cast<size_t>(end - p)));
        const char* e = nl ? nl : end;
        line.assign(p, e);
        p = nl ? nl + 1 : end;
        return true;
    };
    std::string line;
    if (!next_line(line)) throw FormatError(std::string("Matrix Market file is empty: ") + path);
    Header h;
    {
        std::istringstream head(line);
        std::string banner, object, storage, field, symmetry, extra;
        head >> banner >> object >> storage >> field >> symmetry;
        object = lower(object);
        storage = lower(storage);
        field = lower(field);
        symmetry = lower(symmetry);
        if (banner != "%%MatrixMarket" || object != "matrix" || storage != "coordinate" || (head >> extra))
            throw FormatError(std::string("only Matrix Market coordinate matrices are supported: ") + path);
        if (field != "real" && field != "integer" && field != "pattern")
            throw FormatError(std::string("only real, integer, and pattern Matrix Market fields are supported: ") +
                              path);
        if (symmetry == "general") h.sym = kGeneral;
        else if (symmetry == "symmetric") h.sym = kSymmetric;
        else if (symmetry == "skew-symmetric") h.sym = kSkew;
        else if (symmetry == "hermitian") h.sym = kHermitian;
        else throw FormatError("unsupported Matrix Market symmetry: " + symmetry);
        h.pattern = field == "pattern";
    }
    do {
        if (!next_line(line)) throw FormatError(std::string("Matrix Market file has no size line: ") + path);
    } while (blank_or_comment(line.data(), line.data() + line.size()));
    {
        std::istringstream dims(line);
        std::string extra;
        long long e = 0;
        if (!(dims >> h.rows >> h.cols >> e) || h.rows <= 0 || h.cols <= 0 || e < 0 || (dims >> extra))
            throw FormatError(std::string("invalid Matrix Market dimensions: ") + path);
        h.entries = e;
    }
    if (h.sym != kGeneral && h.rows != h.cols)
        throw FormatError("Matrix Market symmetric storage requires a square matrix: " + std::string(path));

    // entry lines: one chunk per thread, cut at line starts
    const unsigned threads = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    const size_t body = static_cast<size_t>(end - p);
    std::vector<const char*> cut{p};
    for (unsigned t = 1; t < threads; ++t) {
        const char* q = p + body * t / threads;
        if (q < cut.back()) q = cut.back();
        const char* nl = q < end ? static_cast<const char*>(std::memchr(q, '\n', static_cast<size_t>(end - q))) : nullptr;
        cut.push_back(nl ? nl + 1 : end);
    }
    cut.push_back(end);
    std::vector<Chunk> chunks(cut.size() - 1);
    std::vector<std::thread> pool;
    for (size_t t = 0; t + 1 < cut.size(); ++t)
        pool.emplace_back([&, t] { parse_chunk(cut[t], cut[t + 1], h, chunks[t]); });
    for (auto& th : pool) th.join();
    // the reference reads exactly `entries` entry lines, then allows only comments
    int64_t seen = 0;
    for (const Chunk& c : chunks) {
        if (c.error_line >= 0 && seen + c.error_line < h.entries) throw FormatError(c.error + ": " + path);
        seen += c.data_lines;
        if (seen > h.entries) throw FormatError(std::string("more Matrix Market entries than declared: ") + path);
    }
    if (seen < h.entries) throw FormatError(std::string("unexpected end of Matrix Market entries: ") + path);

    rows = h.rows;
    cols = h.cols;
    rp.assign(static_cast<size_t>(rows) + 1, 0);
    for (const Chunk& c : chunks)
        for (const Entry& e : c.out) ++rp[static_cast<size_t>(e.row) + 1];
    for (int32_t r = 0; r < rows; ++r) rp[r + 1] += rp[r];
    const int64_t nnz = rp[rows];
    ci.resize(static_cast<size_t>(nnz));
    va.resize(static_cast<size_t>(nnz));
    std::vector<int64_t> cursor(rp.begin(), rp.end() - 1);
    for (const Chunk& c : chunks)
        for (const Entry& e : c.out) {
            const int64_t q = cursor[e.row]++;
            ci[q] = e.column;
            va[q] = e.value;
        }
}

}  // namespace

extern "C" spg_status spg_read_matrix_market(const char* path, int32_t out_location, spg_csr_result* C, char* err,
                                            size_t err_len) {
    auto fail = [&](spg_status s, const std::string& m) {
        if (err && err_len) std::snprintf(err, err_len, "%s", m.c_str());
        return s;
    };
    if (!path || !C || (out_location != SPG_HOST && out_location != SPG_DEVICE))
        return fail(SPG_INVALID_ARGUMENT, "bad arguments");
    std::memset(C, 0, sizeof(*C));
    int32_t rows = 0, cols = 0;
    std::vector<int64_t> rp;
    std::vector<int32_t> ci;
    std::vector<double> va;
    try {
        parse_file(path, rows, cols, rp, ci, va);
    } catch (const FormatError& e) {
        return fail(SPG_FORMAT_ERROR, e.what());
    } catch (const std::bad_alloc&) {
        return fail(SPG_OUT_OF_MEMORY, "host allocation failed");
    }
    const int64_t nnz = static_cast<int64_t>(ci.size());
    C->rows = rows;
    C->cols = cols;
    C->nnz = nnz;
    C->location = out_location;
    const size_t brp = sizeof(int64_t) * rp.size(), bci = sizeof(int32_t) * std::max<int64_t>(nnz, 1),
                 bva = sizeof(double) * std::max<int64_t>(nnz, 1);
    if (out_location == SPG_HOST) {
        C->row_ptr = static_cast<int64_t*>(std::malloc(brp));
        C->col = static_cast<int32_t*>(std::malloc(bci));
        C->val = static_cast<double*>(std::malloc(bva));
        if (!C->row_ptr || !C->col || !C->val) {
            std::free(C->row_ptr);
            std::free(C->col);
            std::free(C->val);
            std::memset(C, 0, sizeof(*C));
            return fail(SPG_OUT_OF_MEMORY, "host allocation failed");
        }
        std::memcpy(C->row_ptr, rp.data(), brp);
        if (nnz) {
            std::memcpy(C->col, ci.data(), sizeof(int32_t) * nnz);
            std::memcpy(C->val, va.data(), sizeof(double) * nnz);
        }
        return SPG_OK;
    }
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&C->row_ptr), brp);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&C->col), bci);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&C->val), bva);
    if (e == cudaSuccess) e = cudaMemcpy(C->row_ptr, rp.data(), brp, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz) e = cudaMemcpy(C->col, ci.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz) e = cudaMemcpy(C->val, va.data(), sizeof(double) * nnz, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(C->row_ptr);
        cudaFree(C->col);
        cudaFree(C->val);
        std::memset(C, 0, sizeof(*C));
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? SPG_OUT_OF_MEMORY : SPG_CUDA_ERROR, cudaGetErrorString(e));
    }
    return SPG_OK;
}

extern "C" void spg_csr_release(spg_csr_result* C) {
    if (!C) return;
    if (C->location == SPG_DEVICE) {
        cudaFree(C->row_ptr);
        cudaFree(C->col);
        cudaFree(C->val);
    } else {
        std::free(C->row_ptr);
        std::free(C->col);
        std::free(C->val);
    }
    std::memset(C, 0, sizeof(*C));
}
