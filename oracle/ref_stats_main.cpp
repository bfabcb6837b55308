// Test-only wrapper that builds the reference's Util_Scripts/calc_stats.cpp,
// UNMODIFIED and with its own main, into oracle/_ref/calc_stats (see
// build_ref.sh).  Used to pin the oracle's restatement of the matrix
// statistics; nothing in the product links against it.
//
// The script includes Util/DriverUtil.hpp only for loadMatrixFromFile; that
// header also pulls in the Boost thread-pool classes (not in this image), so
// its include guard is defined first and loadMatrixFromFile is supplied here:
// it reads a triplet file written by the test harness (int32 row_size,
// col_size, nnz, then nnz int32 rows, nnz int32 columns, nnz float64 values).
// Output is switched to 17 significant digits (round-trip exact for doubles)
// before main runs.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include <boost/lexical_cast.hpp>
#include <boost/random/mersenne_twister.hpp>
#include <boost/random/uniform_real_distribution.hpp>

#include "Matrix/Triplet.hpp"

#define PWM_DRIVERUTIL_HPP
namespace pwm {
template <typename T, typename I>
void loadMatrixFromFile(Triplet<T, I>* m, std::string input_file) {
    std::FILE* f = std::fopen(input_file.c_str(), "rb");
    int32_t hdr[3] = {0, 0, 0};
    if (!f || std::fread(hdr, sizeof(int32_t), 3, f) != 3) {
        std::fprintf(stderr, "cannot read %s\n", input_file.c_str());
        std::exit(2);
    }
    const size_t n = (size_t)hdr[2];
    std::vector<int32_t> r(n), c(n);
    std::vector<double> v(n);
    if (std::fread(r.data(), sizeof(int32_t), n, f) != n || std::fread(c.data(), sizeof(int32_t), n, f) != n ||
        std::fread(v.data(), sizeof(double), n, f) != n) {
        std::fprintf(stderr, "short triplet file %s\n", input_file.c_str());
        std::exit(2);
    }
    std::fclose(f);
    m->row_size = (I)hdr[0];
    m->col_size = (I)hdr[1];
    m->nnz = (I)hdr[2];
    m->row_coord = new I[n];
    m->col_coord = new I[n];
    m->data = new T[n];
    for (size_t k = 0; k < n; ++k) {
        m->row_coord[k] = (I)r[k];
        m->col_coord[k] = (I)c[k];
        m->data[k] = (T)v[k];
    }
}
}  // namespace pwm

namespace {
struct SeventeenDigits {
    SeventeenDigits() { std::cout << std::setprecision(17); }
} g_digits;
}  // namespace

#include "Util_Scripts/calc_stats.cpp"
