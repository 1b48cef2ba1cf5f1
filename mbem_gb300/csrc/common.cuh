// Shared definitions for the mbem_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mbem_gb300.h"

#define MBEM_PI 3.14159265358979323846

namespace mbem {

// Records the last error message for mbem_last_error(); returns `code`.
int set_error(int code, const char* fmt, ...);

// Counts `n_launched` kernel launches and maps the launch status of the last
// kernel to an mbem status.
int launch_status(const char* what, int n_launched = 1);

// Counts kernel launches whose status is checked later.
void count_launches(int n);

// z = M^-1 r for the FGMRES preconditioners (kind 1 block-Jacobi, 2 learned,
// 3 BF16 inner solve).
int bj_apply(const mbem_block_jacobi* bj, const double* r, double* z, cudaStream_t st);
// y = alpha A x + beta y (FP64 row-major at ld)
int dgemv(const double* A, int64_t ld, int64_t n_rows, int64_t n_cols, const double* x, double alpha,
          double beta, double* y, cudaStream_t st);
int precond_apply(int kind, const void* state, const double* r, double* z, cudaStream_t st);
int nn_precond_apply(const void* state, const double* r, double* z, cudaStream_t st);

// Nodal (P1/P2) drivers behind the public entry points when order > 0.
// kind for nodal_matrix: 0 T direct, 1 U direct, 2 T basis, 3 U basis;
// for nodal_contract: 0 T disp, 1 U disp, 2 + MBEM_STRESS_* for stress.
int nodal_matrix(int kind, const double* x, int64_t nf, const double* tv, const double* normals,
                 const double* eps, int64_t ns, const double* coeffs, int order, double alpha,
                 int accumulate, double* out, int64_t ld, void* stream);
// FP64 elastic (DD minus eigen) stress of listed (observer, source) pairs of a
// nodal slip density, nine components per pair (the near pairs of a readout);
// with out_eig, also the pairs' eigenstress.
int nodal_pairs_stress(const double* x, const double* tv, const double* normals, const double* eps,
                       const double* density, double mu, double lam, int order, const int64_t* pair_obs,
                       const int32_t* pair_src, int64_t n_pairs, double* out, cudaStream_t st,
                       double* out_eig = nullptr);
// FP64 traction blocks of listed (field point, source) pairs of an order-0
// source patch, added into out (ld) at columns 3 s .. 3 s + 2 (nodal.cu).
int traction_pairs(const double* x_field, const double* n_field, int64_t n_pts, const double* tri_verts,
                   const double* normals, const double* eps, int64_t n_src, double mu, double lam, int which,
                   double alpha, const int64_t* rowptr, const int64_t* cols, int64_t nnz, double* out, int64_t ld,
                   cudaStream_t st);
int nodal_contract(int kind, const double* x, int64_t nf, const double* tv, const double* normals,
                   const double* eps, int64_t ns, const double* density, const double* coeffs,
                   double mu, double lam, int order, double alpha, int accumulate, double* out,
                   void* stream);

// y = A x for the mixed operator; xh, xl: n floats each (scratch).
int mixed_matvec(const mbem_mixed_operator* op, const double* x, double* y, float* xh, float* xl,
                 cudaStream_t st);

// y = A16 x + near blocks x (BF16 far field, FP32 sums; FP64 near blocks);
// xf: n_cols floats of scratch (16-byte aligned). stop: an optional device
// flag; when set as the kernels start they return without work.
int bf16_matvec(const uint16_t* A16, int64_t ld16, int64_t n_rows, int64_t n_cols, int n_near,
                const mbem_near_blocks* near, const double* x, double* y, float* xf, cudaStream_t st,
                const int* stop = nullptr);
// z = the BF16 inner GMRES solve of r (precond kind 3).
int inner_bf16_apply(const void* state, const double* r, double* z, cudaStream_t st);

// The rank-b (b <= 64) update of a blocked Gauss-Jordan inverse of the FP32 n x n
// M at ld: M[i, j] -= M[i, K] M[K, j] for i, j outside K = [k0, k0 + b), on the
// tensor cores (six BF16 piece products); Ls, Us: n x 384 BF16 each (scratch).
int gj_block_update_tc(float* M, int64_t n, int64_t ld, int64_t k0, int b, uint16_t* Ls, uint16_t* Us,
                       cudaStream_t st);
// C[M x N] -= A[M x K] B[N x K]^T on the tensor cores (BF16 operands, FP32 C).
int gemm_bf16_sub(const void* A, int64_t lda, const void* Bt, int64_t ldb, int64_t M, int64_t N, int64_t K, float* C,
                  int64_t ldc, cudaStream_t st);
// MBEM_ERR_WAIT if a tensor-core wait gave up since the last check (synchronises).
int tc_gemm_check(cudaStream_t st);

// MBEM_ERR_WAIT if a bounded pipeline wait of the mixed matvec gave up since
// the last check; synchronises `st`.
int mixed_wait_check(cudaStream_t st);

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t lmin(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t lmax(int64_t a, int64_t b) { return a > b ? a : b; }

}  // namespace mbem

#define MBEM_REQUIRE(cond, code, ...)                      \
    do {                                                   \
        if (!(cond)) return mbem::set_error((code), __VA_ARGS__); \
    } while (0)

namespace mbem {

// The u-slot ranges (offset, length) whose rigid translations are deflated.
struct URanges {
    int64_t off[8];
    int64_t len[8];
    int n;
};

inline int make_ranges(const int64_t* r, int nr, URanges& ur) {
    MBEM_REQUIRE(nr >= 0 && nr <= 8, MBEM_ERR_ARG, "at most 8 u-slot ranges (got %d)", nr);
    ur.n = nr;
    for (int q = 0; q < nr; q++) {
        ur.off[q] = r[2 * q];
        ur.len[q] = r[2 * q + 1];
        MBEM_REQUIRE(ur.off[q] >= 0 && ur.len[q] >= 0 && ur.len[q] % 3 == 0, MBEM_ERR_ARG,
                     "bad u-slot range (%lld, %lld)", (long long)ur.off[q], (long long)ur.len[q]);
    }
    return MBEM_OK;
}

}  // namespace mbem
