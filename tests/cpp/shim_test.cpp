// The C++ drop-in layer (include/spgemm_gb300.hpp) used the way the reference's
// host code uses its multiply: with the reference's CsrMatrix layout, its
// known answers (spgemm_serial_smoke.cpp:65-67, spgemm_validation_smoke.cpp:
// 153-155, trident_accumulator_memory.cpp:40-60) and its exception types.
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "spgemm_gb300.hpp"

#ifdef SPG_REFERENCE_CSR
// The reference's own type (src/common/csr_matrix.hpp:43-49), where its tree is
// on the include path.
#include "csr_matrix.hpp"
#else
struct CsrMatrix {  // the layout of src/common/csr_matrix.hpp:43-49
    int rows = 0;
    int cols = 0;
    std::vector<int64_t> rowPtr;
    std::vector<int> columnIndices;
    std::vector<double> values;
};
#endif

// The substitution a Trident build makes for its accumulator
// (src/trident/common/matrix_blocks.hpp:23-32).
namespace trident {
using LocalAccumulator = spgemm_gb300::LocalAccumulator<CsrMatrix>;
}

#define REQUIRE(x)                                                   \
    do {                                                             \
        if (!(x)) {                                                  \
            std::fprintf(stderr, "FAILED: %s (line %d)\n", #x, __LINE__); \
            return 1;                                                \
        }                                                            \
    } while (0)

int main() {
    namespace g = spgemm_gb300;
    const CsrMatrix a{2, 3, {0, 2, 3}, {0, 2, 1}, {1.0, 2.0, 3.0}};
    const CsrMatrix b{3, 2, {0, 1, 2, 3}, {1, 0, 1}, {4.0, 5.0, 6.0}};
    const CsrMatrix c = g::spgemm(a, b);
    REQUIRE(c.rows == 2 && c.cols == 2 && c.rowPtr == (std::vector<int64_t>{0, 1, 2}));
    REQUIRE(c.columnIndices == (std::vector<int>{1, 0}) && c.values == (std::vector<double>{16.0, 15.0}));
    REQUIRE(g::thread_engine().scalarMultiplicationCount(a, b) == 3);

    const CsrMatrix ca{3, 2, {0, 2, 2, 3}, {0, 1, 1}, {1, 1, 2}};
    const CsrMatrix cb{2, 3, {0, 2, 4}, {0, 1, 0, 2}, {1, 2, -1, 3}};
    const CsrMatrix cc = g::spgemm(ca, cb);
    REQUIRE(cc.rowPtr == (std::vector<int64_t>{0, 2, 2, 4}));
    REQUIRE(cc.columnIndices == (std::vector<int>{1, 2, 0, 2}) && cc.values == (std::vector<double>{2, 3, -2, 6}));

    bool caught = false;
    try {
        g::spgemm(a, a);  // 2x3 * 2x3
    } catch (const std::invalid_argument&) {
        caught = true;
    }
    REQUIRE(caught);
    caught = false;
    try {
        const CsrMatrix bad{1, 2, {0, 1}, {5}, {1.0}};
        const CsrMatrix two{2, 2, {0, 1, 2}, {0, 1}, {1.0, 1.0}};
        g::spgemm(bad, two);
    } catch (const std::runtime_error&) {
        caught = true;
    }
    REQUIRE(caught);

    // three stages with cross-stage cancellation and an empty row
    CsrMatrix sa{3, 2, {0, 3, 3, 4}, {1, 0, 1, 0}, {2.0, 1.0, -1.0, 3.0}};
    const CsrMatrix sb{2, 4, {0, 3, 5}, {3, 1, 3, 0, 1}, {2.0, 4.0, -1.0, 5.0, -4.0}};
    {
        trident::LocalAccumulator acc(3, 4);
        acc.addProduct(sa, sb);
        for (auto& v : sa.values) v *= -1.0;
        acc.addProduct(sa, sb);
        for (auto& v : sa.values) v *= -0.5;
        acc.addProduct(sa, sb);
        const CsrMatrix r1 = acc.finish();
        const CsrMatrix r2 = acc.finish();  // finish() is const: same result twice
        const CsrMatrix ref = g::spgemm(sa, sb);
        REQUIRE(r1.rowPtr == ref.rowPtr && r1.columnIndices == ref.columnIndices && r1.values == ref.values);
        REQUIRE(r2.values == r1.values && r1.rowPtr[1] == r1.rowPtr[2]);
        caught = false;
        try {
            acc.addProduct(sb, sa);
        } catch (const std::invalid_argument&) {
            caught = true;
        }
        REQUIRE(caught);
    }
    {
        trident::LocalAccumulator empty(0, 4);
        REQUIRE(empty.finish().rowPtr == std::vector<int64_t>{0});
    }
    // the reference's validation, its Matrix Market reader and a transposition, through the same layer
    {
        const spg_full_report rep = g::validateFull(ca, cb, cc);
        REQUIRE(rep.passed == 1 && rep.partial_passed == 1 && rep.matrices_ok == 1 && rep.rejected == 0);
        CsrMatrix wrong = cc;
        wrong.values[0] += 1.0;
        REQUIRE(g::validateFull(ca, cb, wrong).passed == 0);
        const char* path = "shim_test_matrix.mtx";
        FILE* f = std::fopen(path, "w");
        REQUIRE(f != nullptr);
        std::fprintf(f, "%%%%MatrixMarket matrix coordinate real symmetric\n%% c\n3 3 3\n2 1 1.5D0\n3 3 2\n3 1 -4\n");
        std::fclose(f);
        const CsrMatrix m = g::readMatrixMarket<CsrMatrix>(path);
        REQUIRE(m.rows == 3 && m.rowPtr == (std::vector<int64_t>{0, 2, 3, 5}));
        REQUIRE(m.columnIndices == (std::vector<int>{1, 2, 0, 2, 0}));
        REQUIRE(m.values == (std::vector<double>{1.5, -4.0, 1.5, 2.0, -4.0}));
        // A^T lists each column of A by increasing row: row 2 becomes (0, 2), not the file order (2, 0)
        const CsrMatrix mt = g::transpose(m);
        REQUIRE(mt.rowPtr == (std::vector<int64_t>{0, 2, 3, 5}));
        REQUIRE(mt.columnIndices == (std::vector<int>{1, 2, 0, 0, 2}));
        REQUIRE(mt.values == (std::vector<double>{1.5, -4.0, 1.5, -4.0, 2.0}));
        f = std::fopen(path, "w");
        std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n");
        std::fclose(f);
        caught = false;
        try {
            g::readMatrixMarket<CsrMatrix>(path);
        } catch (const std::runtime_error&) {
            caught = true;
        }
        REQUIRE(caught);
        std::remove(path);
    }
    std::printf("shim_test: PASS\n");
    return 0;
}
