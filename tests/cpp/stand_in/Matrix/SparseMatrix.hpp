// Test stand-in for the reference's operator interface, for machines without
// the reference tree: the same names, members and virtual functions as
// pwm::SparseMatrix (Matrix/SparseMatrix.hpp:13-68) and the fields of
// pwm::Triplet (Matrix/Triplet.hpp:27-45) that a caller of the interface
// uses -- an interface has to match to be a drop-in; the loaders, random
// fill and conversions of the real Triplet are not here.  Where the reference
// tree is present, tests/test_cpp_dropin.py also compiles the drop-in header
// against the real Matrix/SparseMatrix.hpp.
#ifndef PWM_SPARSEMATRIX_HPP
#define PWM_SPARSEMATRIX_HPP

namespace pwm {

template <typename T, typename int_type>
class Triplet {
   public:
    int_type* row_coord = nullptr;
    int_type* col_coord = nullptr;
    T* data = nullptr;
    int_type row_size = 0;
    int_type col_size = 0;
    int_type nnz = 0;
};

template <typename T, typename int_type>
class SparseMatrix {
   protected:
    int_type nor;
    int_type noc;
    int_type nnz;

   public:
    SparseMatrix() {}
    SparseMatrix(int threads) { (void)threads; }
    virtual ~SparseMatrix() {}
    virtual void generatePoissonMatrix(const int_type m, const int_type n, const int partitions) = 0;
    virtual void loadFromTriplets(pwm::Triplet<T, int_type>* input, const int partitions_am) = 0;
    virtual void mv(const T* x, T* y) = 0;
    virtual void powerIteration(T* x, T* y, const int_type it) = 0;
};

}  // namespace pwm

#endif  // PWM_SPARSEMATRIX_HPP
