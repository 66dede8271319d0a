// A C++ caller of include/randblas_gb300.hpp, built by tests/test_cpp_api.py.  Exercises the
// host-side parts (states, distributions, next states) and the argument checks, which fail
// before any device work, so it runs without a GPU.  Prints one line per failed check.
#include <cstdio>
#include <string>

#include "randblas_gb300.hpp"

namespace RB = RandBLAS_GB300;

static int failures = 0;
#define EXPECT(cond)                                                 \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAILED %s (line %d)\n", #cond, __LINE__);   \
            ++failures;                                              \
        }                                                            \
    } while (0)

int main() {
    // RNGState(k): counter 0, key k; incr carries across 32-bit limbs
    const RB::RNGState s(0x100000005ull);
    EXPECT(s.s.key[0] == 5u && s.s.key[1] == 1u && s.s.counter[0] == 0u);
    const RB::RNGState t = s.incr(0xFFFFFFFFull).incr(2);
    EXPECT(t.s.counter[0] == 1u && t.s.counter[1] == 1u);

    // DenseDist(200, 10000): wide, Long axis -> natural RowMajor; next state +200*2500
    const RB::DenseDist D(200, 10000);
    EXPECT(D.dim_major == 10000 && D.dim_minor == 200);
    EXPECT(D.natural_layout == RB::Layout::RowMajor);
    const RB::DenseSkOp<double> S(D, RB::RNGState(0));
    EXPECT(S.next_state.s.counter[0] == 500000u);

    // SparseDist(1024, 2^20, 8): SASO, full_nnz = 8 * 2^20, next state + 2^20 * 8
    const RB::SparseDist SD(1024, 1 << 20, 8);
    EXPECT(SD.full_nnz == 8ll << 20);
    const RB::SparseSkOp<float> SS(SD, RB::RNGState(1));
    EXPECT(SS.next_state.s.counter[0] == (8u << 20));

    // argument checks carry the reference's message text and need no device work
    const RB::DenseSkOp<float> Sf(RB::DenseDist(64, 1000), RB::RNGState(2));
    bool threw = false;
    try {
        RB::sketch_general(RB::Layout::RowMajor, RB::Op::NoTrans, RB::Op::NoTrans, 64, 8, 999,
                           1.0f, Sf, static_cast<const float *>(nullptr), 8, 0.0f,
                           static_cast<float *>(nullptr), 8);
    } catch (const RB::Error &e) {
        threw = std::string(e.what()).find("was required, but did not hold") != std::string::npos;
    }
    EXPECT(threw);
    threw = false;
    try {  // lda < n for row-major op(A)
        RB::sketch_general(RB::Layout::RowMajor, RB::Op::NoTrans, RB::Op::NoTrans, 64, 8, 1000,
                           1.0f, Sf, 0, 0, static_cast<const float *>(nullptr), 7, 0.0f,
                           static_cast<float *>(nullptr), 8);
    } catch (const RB::Error &e) {
        threw = e.code == RBG_ERROR_INVALID_ARGUMENT &&
                std::string(e.what()).find("in function lskge3") != std::string::npos;
    }
    EXPECT(threw);
    threw = false;
    try {  // sketch_symmetric checks A before any device work (here: A missing)
        RB::sketch_symmetric(RB::Layout::RowMajor, 1.0f, Sf, static_cast<const float *>(nullptr),
                             1000, 0.0f, static_cast<float *>(nullptr), 1000);
    } catch (const RB::Error &e) {
        threw = std::string(e.what()).find("A must not be NULL") != std::string::npos;
    }
    EXPECT(threw);
    threw = false;
    try {  // random_csr's density check (random_matrix.hh:142) fails before any device work
        RB::RandomSparse R(RB::SparseFormat::CSR, 4, 4, 1.5, RB::RNGState(1));
    } catch (const RB::Error &e) {
        threw = std::string(e.what()).find("density >= 0.0 && density <= 1.0") !=
                    std::string::npos &&
                std::string(e.what()).find("in function random_csr") != std::string::npos;
    }
    EXPECT(threw);
    // conversions: what needs no device work (an empty sort request, a one-entry sort state,
    // the reference's size checks) runs on the host
    EXPECT(RB::coo_arrays_determine_sort<int64_t>(1, nullptr, nullptr) == RB::NonzeroSort::CSC);
    RB::coo_arrays_apply_sort<float, int64_t>(RB::NonzeroSort::None, 5, nullptr, nullptr,
                                              nullptr);
    threw = false;
    try {
        RB::sorted_idxs_to_compressed_ptr<int64_t, int64_t>(0, nullptr, -1, nullptr);
    } catch (const RB::Error &e) {
        threw = std::string(e.what()).find("in function sorted_idxs_to_compressed_ptr") !=
                std::string::npos;
    }
    EXPECT(threw);
    // sparse data: CSR data with an offset, and a sketch_sparse whose data does not match
    // op(A)'s size, fail with the reference's messages before any device work
    {
        int64_t rowptr[7] = {0, 0, 0, 0, 0, 0, 0};
        RB::CSRMatrix<double> A(6, 20, 0, nullptr, rowptr, nullptr);
        threw = false;
        try {
            RB::sparse_data::left_spmm(RB::Layout::ColMajor, RB::Op::NoTrans, RB::Op::NoTrans,
                                       6, 4, 20, 1.0, A, 1, 0, static_cast<const double *>(nullptr),
                                       20, 0.0, static_cast<double *>(nullptr), 6);
        } catch (const RB::Error &e) {
            threw = std::string(e.what()) ==
                    "(ro_a == 0) was required, but did not hold, in function left_spmm";
        }
        EXPECT(threw);
        threw = false;
        try {  // spmm's right form: op(B) = A^T must be n x d = 20 x 6, CSR A is 6 x 20 -> ok;
               // ldc too small for the m x d row-major C
            RB::spmm(RB::Layout::RowMajor, RB::Op::NoTrans, RB::Op::Trans, 4, 6, 20, 1.0,
                     static_cast<const double *>(nullptr), 20, A, 0.0,
                     static_cast<double *>(nullptr), 5);
        } catch (const RB::Error &e) {
            threw = std::string(e.what()) ==
                    "(ldc >= d) was required, but did not hold, in function left_spmm";
        }
        EXPECT(threw);
        RB::DenseSkOp<double> Sd(RB::DenseDist(10, 30), RB::RNGState(2));
        threw = false;
        try {
            RB::sketch_sparse(RB::Layout::RowMajor, RB::Op::NoTrans, RB::Op::NoTrans, 10, 6, 30,
                              1.0, Sd, 0, 0, A, 0.0, static_cast<double *>(nullptr), 6);
        } catch (const RB::Error &e) {
            threw = std::string(e.what()).find("was required, but did not hold") !=
                    std::string::npos;
        }
        EXPECT(threw);
    }
    std::printf("%s\n", failures ? "FAILED" : "ok");
    return failures ? 1 : 0;
}
