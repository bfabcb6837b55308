/*
 * CudaSparseMatrix.hpp -- header-only C++ drop-in classes for the reference's
 * operator interface pwm::SparseMatrix<T, int_type> (Matrix/SparseMatrix.hpp:
 * 13-68), backed by libpwmgpu (include/pwmgpu.h).
 *
 *   pwm::CRSCuda<T, int_type>       merge-path CRS on the GPU (beside CRS_Merge)
 *   pwm::CSBCuda<T, int_type>       CSB on the GPU            (beside CSB)
 *   pwm::BlockCOHCuda<T, int_type>  CO-H on the GPU           (beside BlockCOH)
 *
 * Include it after the reference's Matrix/SparseMatrix.hpp (which brings
 * pwm::Triplet).  T must be double; int_type any 32-bit integer type (int,
 * unsigned int, uint32_t: the instantiations the reference uses,
 * Util/Constants.hpp:32,38 and Tests/poisson.cpp:28,146).  Calls are
 * synchronous like the reference's: y is final when mv returns.  A failing
 * call throws std::runtime_error with pwmgpu_last_error()'s message (the
 * reference asserts instead, CRS.hpp:119).  Loading again frees the previous
 * matrix (the reference leaks it).
 */
#ifndef PWMGPU_CUDA_SPARSE_MATRIX_HPP
#define PWMGPU_CUDA_SPARSE_MATRIX_HPP

#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>

#include "../pwmgpu.h"

namespace pwm {

template <typename T, typename int_type, int Format>
class CudaSparseMatrix : public SparseMatrix<T, int_type> {
    static_assert(std::is_same<T, double>::value, "the GPU classes compute in double");
    static_assert(sizeof(int_type) == 4 && std::is_integral<int_type>::value, "32-bit index types only");

   public:
    // threads: the reference's thread count (-1 = all, CRS_Merge.hpp:69-76);
    // it sets the CO-H partition count, the other formats ignore it.
    explicit CudaSparseMatrix(int threads) : SparseMatrix<T, int_type>(threads) {
        if (threads == -1) threads = (int)std::thread::hardware_concurrency();
        if (threads < 1) threads = 1;
        check(pwmgpu_create(Format, threads, &h_), "pwmgpu_create");
    }
    ~CudaSparseMatrix() override { pwmgpu_destroy(h_); }
    CudaSparseMatrix(const CudaSparseMatrix&) = delete;
    CudaSparseMatrix& operator=(const CudaSparseMatrix&) = delete;

    // SparseMatrix.hpp:41
    void generatePoissonMatrix(const int_type m, const int_type n, const int partitions) override {
        (void)partitions;
        check(pwmgpu_generate_poisson(h_, (int32_t)m, (int32_t)n), "generatePoissonMatrix");
        sync_dims();
    }

    // SparseMatrix.hpp:48 -- sorts the triplet in place, like TripletToCRS.hpp:139-142
    void loadFromTriplets(pwm::Triplet<T, int_type>* input, const int partitions_am) override {
        (void)partitions_am;
        check(pwmgpu_load_triplets(h_, (int32_t)input->row_size, (int32_t)input->col_size, (int32_t)input->nnz,
                                   reinterpret_cast<int32_t*>(input->row_coord),
                                   reinterpret_cast<int32_t*>(input->col_coord), input->data),
              "loadFromTriplets");
        sync_dims();
    }

    // SparseMatrix.hpp:57
    void mv(const T* x, T* y) override { check(pwmgpu_mv(h_, x, y), "mv"); }

    // SparseMatrix.hpp:66 -- the result is in x for even it, in y for odd
    void powerIteration(T* x, T* y, const int_type it) override {
        check(pwmgpu_power(h_, x, y, (int32_t)it), "powerIteration");
    }

    // ---- GPU extras (no counterpart in the reference interface) ----
    // y = A x on device arrays, asynchronous on the handle's stream
    void mv_device(const T* dx, T* dy) { check(pwmgpu_mv_device(h_, dx, dy), "mv_device"); }
    // power solve to ||Au - lambda u|| / |lambda| <= tol (merge format)
    pwmgpu_solve_info solve(T* x, int max_it, double tol, int precision = PWMGPU_PREC_F64) {
        pwmgpu_solve_info info{};
        check(pwmgpu_solve(h_, x, max_it, tol, precision, &info), "solve");
        return info;
    }
    pwmgpu_matrix* handle() const { return h_; }

   private:
    pwmgpu_matrix* h_ = nullptr;

    void sync_dims() {
        int32_t nor = 0, noc = 0;
        int64_t nnz = 0;
        check(pwmgpu_dims(h_, &nor, &noc, &nnz), "pwmgpu_dims");
        this->nor = (int_type)nor;
        this->noc = (int_type)noc;
        this->nnz = (int_type)nnz;
    }
    static void check(int rc, const char* what) {
        if (rc != PWMGPU_OK) throw std::runtime_error(std::string(what) + ": " + pwmgpu_last_error());
    }
};

template <typename T, typename int_type>
using CRSCuda = CudaSparseMatrix<T, int_type, PWMGPU_FMT_MERGE>;
template <typename T, typename int_type>
using CSBCuda = CudaSparseMatrix<T, int_type, PWMGPU_FMT_CSB>;
template <typename T, typename int_type>
using BlockCOHCuda = CudaSparseMatrix<T, int_type, PWMGPU_FMT_COH>;
// format autotuned per matrix class (pwmgpu_tuning_info on handle())
template <typename T, typename int_type>
using AutoCuda = CudaSparseMatrix<T, int_type, PWMGPU_FMT_AUTO>;

}  // namespace pwm

#endif  // PWMGPU_CUDA_SPARSE_MATRIX_HPP
