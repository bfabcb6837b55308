// Test-only harness around the UNMODIFIED reference headers (KobeBergmans/Thesis_SPMV).
//
// This file is oracle infrastructure: it is compiled in the development
// container only, straight from the reference tree (see build_ref.sh), into
// oracle/_ref/libpwmref.so.  It is used to pin the C restatement in
// oracle/oracle.c and to generate the golden fixtures in tests/golden/.
// Nothing in the product links against it.
//
// The reference keeps its arrays protected: the harness opens them with a
// test-only access macro after all standard headers are in.  The two private
// functions it needs (CRS_Merge::searchPathOnDiag, BlockCOH::rowColToHilbert)
// are reached through the explicit-instantiation access idiom below
// (`private` cannot be redefined: OpenMP's private(...) clause uses the word).
#include <algorithm>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>
#include <sys/stat.h>
#include <omp.h>

#include <boost/lexical_cast.hpp>
#include <boost/random/mersenne_twister.hpp>
#include <boost/random/uniform_real_distribution.hpp>

#define protected public
#include "Matrix/Triplet.hpp"
#include "Matrix/SparseMatrix.hpp"
#include "Matrix/CRS.hpp"
#include "Env_Implementations/CRSOMP.hpp"
#include "SOA_Implementations/CRS_Merge.hpp"
#include "SOA_Implementations/CSB.hpp"
#include "SOA_Implementations/BlockCOH.hpp"
#undef protected

// Explicit instantiation may name private members; the friend function then
// hands out the member pointer.
template <typename Tag, typename Tag::type M>
struct Rob { friend typename Tag::type get(Tag) { return M; } };
struct MergeSearchTag {
    typedef std::tuple<int, int> (pwm::CRS_Merge<double, int>::*type)(const int, const int*);
    friend type get(MergeSearchTag);
};
template struct Rob<MergeSearchTag, &pwm::CRS_Merge<double, int>::searchPathOnDiag>;
struct HilbertTag {
    typedef int (pwm::BlockCOH<double, int>::*type)(const int, int, int);
    friend type get(HilbertTag);
};
template struct Rob<HilbertTag, &pwm::BlockCOH<double, int>::rowColToHilbert>;

typedef pwm::SparseMatrix<double, int> SM;
typedef pwm::Triplet<double, int> TR;

extern "C" {

// ---- Triplet loaders / generators (Matrix/Triplet.hpp) ----
void* ref_triplet_new() { TR* t = new TR(); t->row_coord = nullptr; t->col_coord = nullptr; t->data = nullptr; t->nnz = 0; return t; }
void ref_triplet_delete(void* h) { delete (TR*)h; }
void ref_triplet_load_mm(void* h, const char* fn, int has_data, int symmetric, int random_fill) {
    ((TR*)h)->loadFromMM(fn, has_data != 0, symmetric != 0, random_fill != 0);
}
void ref_triplet_load_bin(void* h, const char* fn, int mat_size, int symmetric, int random_vals) {
    ((TR*)h)->loadFromBin(fn, mat_size, symmetric != 0, random_vals != 0);
}
void ref_triplet_poisson(void* h, int m, int n) { ((TR*)h)->generatePoisson(m, n); }
void ref_triplet_set(void* h, int nor, int noc, int nnz, const int* r, const int* c, const double* v) {
    TR* t = (TR*)h;
    delete[] t->row_coord; delete[] t->col_coord; delete[] t->data;
    t->row_size = nor; t->col_size = noc; t->nnz = nnz;
    t->row_coord = new int[nnz]; t->col_coord = new int[nnz]; t->data = new double[nnz];
    std::copy(r, r + nnz, t->row_coord); std::copy(c, c + nnz, t->col_coord); std::copy(v, v + nnz, t->data);
}
int ref_triplet_info(void* h, int* nor, int* noc) { TR* t = (TR*)h; *nor = t->row_size; *noc = t->col_size; return t->nnz; }
void ref_triplet_get(void* h, int* r, int* c, double* v) {
    TR* t = (TR*)h;
    std::copy(t->row_coord, t->row_coord + t->nnz, r); std::copy(t->col_coord, t->col_coord + t->nnz, c);
    std::copy(t->data, t->data + t->nnz, v);
}

// ---- Matrix classes (method numbers as in Util/DriverUtil.hpp selectType) ----
void* ref_matrix_new(int method, int threads) {
    switch (method) {
        case 1: return (SM*)new pwm::CRS<double, int>(threads);
        case 2: return (SM*)new pwm::CRSOMP<double, int>(threads);
        case 8: return (SM*)new pwm::CRS_Merge<double, int>(threads);
        case 9: return (SM*)new pwm::CSB<double, int>(threads);
        case 10: return (SM*)new pwm::BlockCOH<double, int>(threads);
        default: return nullptr;
    }
}
void ref_matrix_delete(void* h) { delete (SM*)h; }
void ref_generate_poisson(void* h, int m, int n, int partitions) { ((SM*)h)->generatePoissonMatrix(m, n, partitions); }
void ref_load_triplets(void* h, void* trip, int partitions) { ((SM*)h)->loadFromTriplets((TR*)trip, partitions); }
void ref_mv(void* h, const double* x, double* y) { ((SM*)h)->mv(x, y); }
void ref_power(void* h, double* x, double* y, int it) { ((SM*)h)->powerIteration(x, y, it); }
int ref_dims(void* h, int* nor, int* noc) { SM* s = (SM*)h; *nor = s->nor; *noc = s->noc; return s->nnz; }

// CRS family peek (methods 1, 2, 8 share the same three arrays)
void ref_crs_get(void* h, int method, int* row_start, int* col_ind, double* data) {
    SM* s = (SM*)h;
    int *rs, *ci; double* d;
    if (method == 1) { auto* m = (pwm::CRS<double, int>*)s; rs = m->row_start; ci = m->col_ind; d = m->data_arr; }
    else { auto* m = (pwm::CRSOMP<double, int>*)s; rs = m->row_start; ci = m->col_ind; d = m->data_arr; }
    std::copy(rs, rs + s->nor + 1, row_start); std::copy(ci, ci + s->nnz, col_ind); std::copy(d, d + s->nnz, data);
}

// CRS_Merge::searchPathOnDiag (SOA_Implementations/CRS_Merge.hpp:42-62)
void ref_merge_search(void* h, int diagonal, int* a, int* b) {
    auto* m = (pwm::CRS_Merge<double, int>*)(SM*)h;
    auto t = (m->*get(MergeSearchTag()))(diagonal, m->row_start + 1);
    *a = std::get<0>(t); *b = std::get<1>(t);
}

// CSB arrays (SOA_Implementations/CSB.hpp:34-59)
void ref_csb_info(void* h, int* beta, int* block_bits, int* hblocks, int* vblocks, int* balanced) {
    auto* m = (pwm::CSB<double, int>*)(SM*)h;
    *beta = m->beta; *block_bits = m->block_bits; *hblocks = m->horizontal_blocks; *vblocks = m->vertical_blocks;
    *balanced = m->balanced_block_rows ? 1 : 0;
}
void ref_csb_get(void* h, uint32_t* ind, double* data, int* blk_ptr) {
    auto* m = (pwm::CSB<double, int>*)(SM*)h;
    std::copy(m->ind, m->ind + m->nnz, ind); std::copy(m->data, m->data + m->nnz, data);
    std::copy(m->blk_ptr, m->blk_ptr + (size_t)m->horizontal_blocks * m->vertical_blocks + 1, blk_ptr);
}

// BlockCOH arrays (SOA_Implementations/BlockCOH.hpp:27-67)
int ref_coh_threads(void* h) { return ((pwm::BlockCOH<double, int>*)(SM*)h)->threads; }
void ref_coh_thread_info(void* h, int pid, int* row_start, int* beta, int* block_bits, int* hblocks, int* vblocks,
                         int* tnnz, int* tblocks, int* n_row_jump, int* n_row_jump_block) {
    auto* m = (pwm::BlockCOH<double, int>*)(SM*)h;
    *row_start = m->thread_row_start[pid]; *beta = m->beta[pid]; *block_bits = m->block_bits[pid];
    *hblocks = m->horizontal_blocks[pid]; *vblocks = m->vertical_blocks[pid];
    *tnnz = m->thread_nnz[pid]; *tblocks = m->thread_blocks[pid];
    // Count the row jumps actually used by replaying the decode of BlockCOH::blockMult / mv.
    int rj = 0, ci = 0;
    for (int b = 0; b < m->thread_blocks[pid]; ++b) {
        int col = m->col_jump[pid][ci]; rj++;
        for (int i = 0; i < m->block_nnz[pid][b] - 1; ++i) {
            ci++; col += m->col_jump[pid][ci];
            if (col >= m->beta[pid]) { col -= m->beta[pid]; rj++; }
        }
        ci++;
    }
    *n_row_jump = rj;
    int rjb = 1, bc = m->col_jump_block[pid][0];
    for (int b = 1; b < m->thread_blocks[pid]; ++b) {
        bc += m->col_jump_block[pid][b];
        if (bc >= m->horizontal_blocks[pid]) { bc -= m->horizontal_blocks[pid]; rjb++; }
    }
    *n_row_jump_block = rjb;
}
void ref_coh_thread_get(void* h, int pid, uint16_t* row_jump, int n_row_jump, uint16_t* col_jump, double* data,
                        int* block_nnz, int16_t* row_jump_block, int n_row_jump_block, int16_t* col_jump_block) {
    auto* m = (pwm::BlockCOH<double, int>*)(SM*)h;
    int tn = m->thread_nnz[pid], tb = m->thread_blocks[pid];
    std::copy(m->row_jump[pid], m->row_jump[pid] + n_row_jump, row_jump);
    std::copy(m->col_jump[pid], m->col_jump[pid] + tn, col_jump);
    std::copy(m->data[pid], m->data[pid] + tn, data);
    std::copy(m->block_nnz[pid], m->block_nnz[pid] + tb, block_nnz);
    std::copy(m->row_jump_block[pid], m->row_jump_block[pid] + n_row_jump_block, row_jump_block);
    std::copy(m->col_jump_block[pid], m->col_jump_block[pid] + tb, col_jump_block);
}
// BlockCOH::rowColToHilbert (SOA_Implementations/BlockCOH.hpp:103-114)
int ref_hilbert(int size, int row, int col) {
    pwm::BlockCOH<double, int> m(1);
    int r = (m.*get(HilbertTag()))(size, row, col);
    m.threads = 0; m.row_jump = nullptr; m.col_jump = nullptr; m.data = nullptr; m.row_jump_block = nullptr;
    m.col_jump_block = nullptr; m.block_nnz = nullptr; m.thread_row_start = nullptr; m.beta = nullptr;
    m.block_bits = nullptr; m.vertical_blocks = nullptr; m.horizontal_blocks = nullptr; m.thread_nnz = nullptr;
    m.thread_blocks = nullptr;
    return r;
}

// ---- Util/TripletToCRS.hpp:309-385 (TripletToMultipleCRS): the blocks'
// arrays concatenated as orc_triplet_to_multi_crs writes them; the triplet
// arrays are sorted in place as the reference sorts them ----
void ref_multi_crs(int nor, int nnz, int parts, int* r, int* c, double* v, int* first_rows, int* thread_rows,
                   int* rs_all, int* ci_all, double* d_all) {
    std::vector<int*> rs(parts), ci(parts);
    std::vector<double*> d(parts);
    pwm::TripletToMultipleCRS<double, int>(r, c, v, rs.data(), ci.data(), d.data(), parts, thread_rows, first_rows,
                                           nnz, nor);
    int base = 0, k0 = 0;
    for (int p = 0; p < parts; ++p) {
        const int n = rs[p][thread_rows[p]];
        std::copy(rs[p], rs[p] + thread_rows[p] + 1, rs_all + base);
        std::copy(ci[p], ci[p] + n, ci_all + k0);
        std::copy(d[p], d[p] + n, d_all + k0);
        base += thread_rows[p] + 1;
        k0 += n;
        delete[] rs[p];
        delete[] ci[p];
        delete[] d[p];
    }
}
// ---- Util/Poisson.hpp:33-83 with first_row / last_row ----
void ref_fill_poisson_rows(int m, int n, int first_row, int last_row, int* rs, int* ci, double* d) {
    pwm::fillPoisson<double, int>(d, rs, ci, m, n, first_row, last_row);
}

void ref_set_threads(int t) { omp_set_num_threads(t); }
int ref_max_threads() { return omp_get_max_threads(); }
void ref_srand(unsigned s) { srand(s); }
}
