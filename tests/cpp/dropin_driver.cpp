// A driver in the shape of the reference's driver_poisson.cpp / test.cpp,
// using the GPU classes through pwm::SparseMatrix only (methods 12, 13, 14
// and the autotuned 15, next to the reference's 1-10 in
// Util/DriverUtil.hpp:38-84 selectType).
//
//   dropin_driver <method> <m> <n> <it> <out.bin> [u32|int|unsigned]
//
// The last argument picks the index type the classes are instantiated with:
// uint32_t (the drivers' type, Util/Constants.hpp:32,38, the default), int or
// unsigned int (the types Tests/poisson.cpp:28,146 instantiates).
// Writes, as doubles: y = A x (x = 1) for the m x n Poisson matrix, the
// powerIteration result (x = 1, `it` iterations), and y = B x for a seeded
// random triplet B loaded with loadFromTriplets; then checks that the power
// method on a rectangular matrix throws.  The test compares these with the
// oracle.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "Matrix/SparseMatrix.hpp"
#include "pwmgpu/CudaSparseMatrix.hpp"

template <typename I>
static pwm::SparseMatrix<double, I>* select_type(int method, int threads) {
    switch (method) {
        case 12: return new pwm::CRSCuda<double, I>(threads);
        case 13: return new pwm::CSBCuda<double, I>(threads);
        case 14: return new pwm::BlockCOHCuda<double, I>(threads);
        case 15: return new pwm::AutoCuda<double, I>(threads);
        default: return nullptr;  // like selectType's NULL (DriverUtil.hpp:81-82)
    }
}

template <typename I>
static int run(int method, I m, I n, I it, const char* path) {
    std::unique_ptr<pwm::SparseMatrix<double, I>> A(select_type<I>(method, 4));
    if (!A) return 3;
    std::FILE* out = std::fopen(path, "wb");
    if (!out) return 4;
    A->generatePoissonMatrix(m, n, 4);
    const size_t N = (size_t)m * n;
    std::vector<double> x(N, 1.0), y(N, 0.0);
    A->mv(x.data(), y.data());
    std::fwrite(y.data(), sizeof(double), N, out);
    std::fill(x.begin(), x.end(), 1.0);
    std::fill(y.begin(), y.end(), 0.0);
    A->powerIteration(x.data(), y.data(), it);
    std::fwrite(it % 2 == 0 ? x.data() : y.data(), sizeof(double), N, out);

    // a seeded random triplet (LCG), loaded through loadFromTriplets
    const I R = 501, nnz = 4000;
    std::vector<I> rows, cols;
    std::vector<double> vals;
    uint64_t s = 12345;
    auto next = [&]() { s = s * 6364136223846793005ull + 1442695040888963407ull; return (uint32_t)(s >> 33); };
    std::vector<char> seen((size_t)R * R, 0);
    while (rows.size() < nnz) {
        const I r = (I)(next() % (uint32_t)R), c = (I)(next() % (uint32_t)R);
        if (seen[(size_t)r * R + c]) continue;
        seen[(size_t)r * R + c] = 1;
        rows.push_back(r);
        cols.push_back(c);
        vals.push_back((double)(next() % 2000) / 1000.0 - 1.0);
    }
    pwm::Triplet<double, I> t;
    t.row_coord = rows.data();
    t.col_coord = cols.data();
    t.data = vals.data();
    t.row_size = R;
    t.col_size = R;
    t.nnz = nnz;
    std::unique_ptr<pwm::SparseMatrix<double, I>> B(select_type<I>(method, 4));
    B->loadFromTriplets(&t, 4);
    std::vector<double> xb(R), yb(R);
    for (I i = 0; i < R; ++i) xb[i] = 1.0 + (double)(i % 7);
    B->mv(xb.data(), yb.data());
    std::fwrite(yb.data(), sizeof(double), R, out);
    // the triplet comes back sorted (TripletToCRS.hpp:139-142): write it too
    std::fwrite(rows.data(), sizeof(I), nnz, out);
    std::fwrite(cols.data(), sizeof(I), nnz, out);
    std::fwrite(vals.data(), sizeof(double), nnz, out);

    // powerIteration on a rectangular matrix throws (CRS.hpp:119 asserts)
    pwm::Triplet<double, I> r2;
    I rr[1] = {0}, cc[1] = {5};
    double vv[1] = {1.0};
    r2.row_coord = rr;
    r2.col_coord = cc;
    r2.data = vv;
    r2.row_size = 3;
    r2.col_size = 7;
    r2.nnz = 1;
    std::unique_ptr<pwm::SparseMatrix<double, I>> Cm(select_type<I>(method, 4));
    Cm->loadFromTriplets(&r2, 4);
    int threw = 0;
    std::vector<double> a(7, 1.0), b(7, 0.0);
    try {
        Cm->powerIteration(a.data(), b.data(), 2);
    } catch (const std::runtime_error&) {
        threw = 1;
    }
    std::fclose(out);
    std::printf("threw=%d\n", threw);
    return threw ? 0 : 5;
}

int main(int argc, char** argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s <method> <m> <n> <it> <out.bin> [u32|int|unsigned]\n", argv[0]);
        return 2;
    }
    const int method = std::atoi(argv[1]);
    const int m = std::atoi(argv[2]), n = std::atoi(argv[3]), it = std::atoi(argv[4]);
    const std::string type = argc > 6 ? argv[6] : "u32";
    if (type == "int") return run<int>(method, m, n, it, argv[5]);
    if (type == "unsigned") return run<unsigned int>(method, (unsigned)m, (unsigned)n, (unsigned)it, argv[5]);
    if (type == "u32") return run<uint32_t>(method, (uint32_t)m, (uint32_t)n, (uint32_t)it, argv[5]);
    std::fprintf(stderr, "unknown index type %s\n", type.c_str());
    return 2;
}
