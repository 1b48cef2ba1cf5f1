/*
 * mbem_gb300 C ABI: the GB300 (sm_103a) hot path of the mollified boundary
 * element method behind plain pointers and sizes.
 *
 * Conventions for every entry point:
 *  - array arguments are DEVICE pointers to C-contiguous float64 arrays in
 *    the reference's layouts (x_field (Nf,3); tri_verts (Ns,3,3) vertex
 *    major; normals (Ns,3); eps (Ns,); density (K*Ns,3); matrices row-major
 *    (3Nf, 3KNs) with block (3f+i, 3(K s+k)+j); stress (Nf,3,3));
 *  - small coefficient vectors (`coeffs`, `shape`, slot ranges) are HOST
 *    pointers;
 *  - `stream` is a cudaStream_t (NULL = legacy default stream); every call
 *    is asynchronous on it unless stated otherwise;
 *  - the return value is an mbem_status; mbem_last_error() describes the
 *    last failure of the calling thread;
 *  - nothing allocates device memory: scratch comes from a caller-provided
 *    workspace whose size the matching *_workspace_size query returns.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the reference project's root).
 */
#ifndef MBEM_GB300_H
#define MBEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MBEM_OK = 0,
    MBEM_ERR_ARG = 1,          /* invalid argument: NULL pointer, bad size, order or kind */
    MBEM_ERR_UNSUPPORTED = 2,  /* a combination the library does not implement */
    MBEM_ERR_CUDA = 3,         /* a CUDA runtime or launch failure */
    MBEM_ERR_WAIT = 4,         /* a bounded device-side wait expired */
    MBEM_ERR_SIZE = 5,         /* a size beyond a stated maximum, or a workspace too small */
    MBEM_ERR_NUMERIC = 6       /* breakdown detected (zero pivot, non-finite value) */
} mbem_status;

/* Kinds of mbem_stress_contract. */
enum {
    MBEM_STRESS_DD = 0,        /* slip -> total stress (tri_nodal.py:1344 dd_stress_contract) */
    MBEM_STRESS_KELVIN = 1,    /* force -> stress (tri_nodal.py:1334 kelvin_stress_contract) */
    MBEM_STRESS_EIGEN = 2,     /* exact eigenstress +C:eps* (tri_nodal.py:1355 eigenstress_contract) */
    MBEM_STRESS_ELASTIC = 3    /* dd minus eigen in one pass (evaluate.py:383-407 _double_layer_stress) */
};

/* Library identity and the last error message of the calling thread. */
int mbem_version(void);
const char* mbem_last_error(void);
/* Kernels this library has launched since it was loaded (all threads). */
unsigned long long mbem_launch_count(void);
/* The FP32 pipe's FMA throughput: 16 independent FFMA chains a thread
 * (packed = 0) or 8 FFMA2 (float2) chains (packed = 1), `iters` steps; the
 * same 32 FLOPs a thread a step either way (bench roofline denominator). */
int mbem_fp32_fma_probe(float* out, int64_t iters, int blocks, int threads, int packed, void* stream);
/* FP64 pipe throughput probe: blocks*threads threads each run 8 independent
 * DFMA chains of `iters` steps (16*iters FLOP per thread); time it with
 * events for the FP64 roofline denominator. No reference counterpart. */
int mbem_fp64_fma_probe(double* out, int64_t iters, int blocks, int threads, void* stream);

/* ---- kernel matrices: src/mbem/kernels/tri_nodal.py:1289-1306 (public
 * drivers) and src/mbem/kernels/tri_kernels.py:547-591 (P0 direct).
 * out(3Nf, 3KNs) at leading dimension ld_out: out = alpha*M (accumulate=0)
 * or out += alpha*M (accumulate=1), so a block lands directly inside a
 * larger system matrix. coeffs: 6 T coefficients (basis.py:58-72 t_coeffs)
 * or 3 U coefficients (basis.py:46-55 u_coeffs). ---------------------- */
int mbem_t_matrix_direct(const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src,
                         const double* coeffs, int order, double alpha, int accumulate,
                         double* out, int64_t ld_out, void* stream);
int mbem_u_matrix_direct(const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* eps, int64_t n_src, const double* coeffs, int order,
                         double alpha, int accumulate, double* out, int64_t ld_out, void* stream);

/* Geometry-only basis stacks (6 or 3, 3Nf, 3KNs), contiguous:
 * tri_nodal.py t_basis_matrices / u_basis_matrices (tri_kernels.py:451-492). */
int mbem_t_basis_matrices(const double* x_field, int64_t n_field, const double* tri_verts,
                          const double* normals, const double* eps, int64_t n_src, int order,
                          double* out, void* stream);
int mbem_u_basis_matrices(const double* x_field, int64_t n_field, const double* tri_verts,
                          const double* eps, int64_t n_src, int order, double* out, void* stream);

/* ---- matrix-free contractions (tri_kernels.py:976-1260; tri_nodal.py
 * :1310-1366). Displacement out (Nf,3); stress out (Nf,3,3). out = alpha*r
 * or out += alpha*r. Sources with an all-zero density are skipped, as the
 * reference does. ------------------------------------------------------ */
int mbem_t_disp_contract(const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src,
                         const double* density, const double* coeffs, int order, double alpha,
                         int accumulate, double* out, void* stream);
int mbem_u_disp_contract(const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* eps, int64_t n_src, const double* density,
                         const double* coeffs, int order, double alpha, int accumulate,
                         double* out, void* stream);
int mbem_stress_contract(int kind, const double* x_field, int64_t n_field,
                         const double* tri_verts, const double* normals, const double* eps,
                         int64_t n_src, const double* density, double mu, double lam, int order,
                         double alpha, int accumulate, double* out, void* stream);

/* ---- traction rows: tri_nodal.py:1370-1404 traction_matrix /
 * basis.py:406-427 assemble_traction_matrix. which: 0 "slip" (total minus
 * eigen), 1 "force", 2 "eigen", 3 "total". ids (Ns,K) int64 DEVICE array
 * scattering element-node columns onto n_cols shared columns; out
 * (3Nf, 3 n_cols) at ld_out, accumulated (out += alpha * rows); an id
 * outside [0, n_cols) contributes nothing. ------------------------------ */
int mbem_traction_matrix(const double* x_field, const double* n_field, int64_t n_pts,
                         const double* tri_verts, const double* normals, const double* eps,
                         int64_t n_src, const int64_t* ids, int64_t n_cols, double mu, double lam,
                         int order, int which, double alpha, double* out, int64_t ld_out,
                         void* stream);

/* The same traction rows (which = "slip", an order-0 source patch) for the
 * mixed operator: far pairs by FP32 quadrature of the point integrand (DD
 * stress minus eigenstress), near pairs (the near list near_rowptr/near_cols
 * of mbem_near_count/mbem_near_fill at near_factor) by the FP64 closed form;
 * out (3 n_pts, 3 n_src) at ld_out, accumulated (out += alpha * rows). */
int mbem_traction_matrix_mixed(const double* x_field, const double* n_field, int64_t n_pts,
                               const double* tri_verts, const double* normals, const double* eps, int64_t n_src,
                               double mu, double lam, double near_factor, double alpha, const int64_t* near_rowptr,
                               const int64_t* near_cols, int64_t nnz, double* out, int64_t ld_out, void* stream);

/* ---- dense-system helpers of the calibrated dense backend
 * (src/mbem/backends/dense.py:480-528). ------------------------------- */

/* out[r, j] (+)= alpha * sum_c A[r, 3c + j] for c < n_col_nodes: the
 * calibration row sums (dense.py:497-500 rowsum, equations.py:512-537). */
int mbem_block_rowsum3(const double* A, int64_t ld, int64_t n_rows, int64_t n_col_nodes,
                       double alpha, int accumulate, double* out, void* stream);

/* A[r0 + 3c + a, c0 + 3(K s + k) + b] += shape[kc*K + k] * D[c, a, b] for
 * c = K s + kc (equations.py:566-582 add_block_diagonal). A points at the
 * block's top-left corner; shape is a HOST (K,K) array. */
int mbem_add_block_diagonal(double* A, int64_t ld, const double* D, int64_t n_c, int K,
                            const double* shape, void* stream);

/* In place, rows (3c, 3c+1, 3c+2) of A (n_cols wide, at ld) and entries
 * (3c..3c+2) of b (may be NULL) become F_c times themselves, F = frames
 * (n_nodes, 3, 3) DEVICE: a traction fault's Cartesian rows into its row
 * frame (equations.py:443-473 apply_fault_rows). A and b point at the
 * fault's first row. */
int mbem_rotate_row_triples(double* A, int64_t ld, int64_t n_cols, double* b, int64_t n_nodes,
                            const double* frames, void* stream);

/* y = alpha * A x + beta * y, FP64 row-major (the dense matvec of
 * la/solver.py:513-520 _as_matvec on an AssembledDense.A). */
int mbem_dgemv(const double* A, int64_t ld, int64_t n_rows, int64_t n_cols, const double* x,
               double alpha, double beta, double* y, void* stream);

/* Y = A X for k right-hand sides (X, Y row-major (n, k)): the multi-RHS
 * refinement product of la/lu.py:210. */
int mbem_dgemm_multi(const double* A, int64_t ld, int64_t n_rows, int64_t n_cols, const double* X,
                     int64_t k, double* Y, void* stream);

/* ---- mixed-precision operator: A = A_far (FP32 dense) + A_near (FP64
 * 3x3 blocks in CSR by field point). It replaces the FP64 AssembledDense.A
 * of backends/dense.py:480-528 in the mixed mode; no reference counterpart
 * beyond that role. ------------------------------------------------- */
typedef struct {
    int64_t row0, col0;      /* offsets of this block in the system's rows / columns */
    int64_t n_field;         /* field points (row blocks of 3 rows) */
    const int64_t* rowptr;   /* (n_field + 1) device */
    const int64_t* cols;     /* (nnz) source index of each near block, device */
    const double* vals;      /* (nnz, 3, 3) device */
} mbem_near_blocks;

typedef struct {
    int64_t n_rows, n_cols;  /* square (the unknowns) for a solve; any shape for a product */
    const float* A32;        /* (n_rows, n_cols) FP32 far field at leading dimension ld32, device */
    int64_t ld32;
    int n_near;
    const mbem_near_blocks* near;  /* HOST array of n_near descriptors */
} mbem_mixed_operator;

/* FP32 far-field block (kernel 0 = T with 6 coeffs, 1 = U with 3) of
 * alpha * M into out (3Nf, 3Ns) at ld_out; near pairs (centroid distance
 * below near_factor * max(eps, mean edge), or below 1.5 longest edge) are
 * written as zeros. near_mask (optional, device, n_field x ceil(Ns/32)
 * uint32) receives one bit per near pair, source s at word s/32, bit s%32. */
int mbem_far_matrix(int kernel, const double* x_field, int64_t n_field, const double* tri_verts,
                    const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                    double near_factor, double alpha, float* out, int64_t ld_out, uint32_t* near_mask,
                    void* stream);
/* The same, also writing out16 = BF16(out) (round to nearest even) at ld16:
 * the inner operator's copy, made by the assembly with no extra pass. */
int mbem_far_matrix_bf16(int kernel, const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                         double near_factor, double alpha, float* out, int64_t ld_out, uint16_t* out16,
                         int64_t ld16, uint32_t* near_mask, void* stream);
/* The same for a nodal source density of order 0/1/2: columns 3 (K s + k) + j
 * (K = 1, 3, 6), node k's block by the far quadrature weighted with its
 * Lagrange shape function; the near mask is per (field point, source). */
int mbem_far_matrix_nodal(int kernel, int order, const double* x_field, int64_t n_field, const double* tri_verts,
                          const double* normals, const double* eps, int64_t n_src, const double* coeffs,
                          double near_factor, double alpha, float* out, int64_t ld_out, uint16_t* out16,
                          int64_t ld16, uint32_t* near_mask, void* stream);
/* FP64 nodal (order 1/2) blocks of the listed near pairs (rowptr/cols by
 * field point over sources, nnz pairs): node k of pair q into
 * vals[(K q + k) * 9 .. + 9], i.e. the near list by nodes (columns K s + k). */
int mbem_near_eval_nodal(int kernel, int order, const double* x_field, int64_t n_field, const double* tri_verts,
                         const double* normals, const double* eps, const int64_t* rowptr, const int64_t* cols,
                         int64_t nnz, const double* coeffs, double alpha, double* vals, void* stream);
/* The calibrated diagonal D (n_field x 3 x 3) of collocation point c = K s + kc
 * added to the near blocks of its element's nodes K s + k with the collocation
 * shape weights shape[kc * K + k]; *missing counts absent self blocks. */
int mbem_near_add_diagonal_nodal(const int64_t* rowptr, const int64_t* cols, double* vals, int64_t n_field,
                                 const double* D, int K, const double* shape, int* missing, void* stream);
/* Near list from that bit mask: rowptr (n_field+1) and nnz on the host
 * (synchronises `stream`), then the source indices in increasing order. */
int mbem_near_mask_count(const uint32_t* mask, int64_t n_field, int64_t n_src, int64_t* rowptr,
                         void* work, size_t work_bytes, int64_t* nnz_host, void* stream);
int mbem_near_mask_fill(const uint32_t* mask, int64_t n_field, int64_t n_src, const int64_t* rowptr,
                        int64_t* cols, void* stream);
/* Near list, pass 1: rowptr (n_field+1) device; nnz returned on the host
 * (the call synchronises `stream`). work >= mbem_near_list_workspace_size. */
size_t mbem_near_list_workspace_size(int64_t n_field);
int mbem_near_count(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                    int64_t n_src, double near_factor, int64_t* rowptr, void* work, size_t work_bytes,
                    int64_t* nnz_host, void* stream);
/* Near list, pass 2: source indices in increasing order per field point. */
int mbem_near_fill(const double* x_field, int64_t n_field, const double* tri_verts, const double* eps,
                   int64_t n_src, double near_factor, const int64_t* rowptr, int64_t* cols, void* stream);
/* FP64 closed-form blocks alpha * M for the near list (kernel as above). */
int mbem_near_eval(int kernel, const double* x_field, int64_t n_field, const double* tri_verts,
                   const double* normals, const double* eps, const int64_t* rowptr, const int64_t* cols,
                   int64_t nnz, const double* coeffs, double alpha, double* vals, void* stream);
/* Calibration row sums of far + near: out (n_rows/3, 3, 3) = sum over
 * column nodes (far in double-float, near in FP64). */
int mbem_mixed_rowsum3(const float* A32, int64_t ld, int64_t n_rows, int64_t n_col_nodes,
                       const int64_t* rowptr, const double* vals, double* out, void* stream);
/* Adds D (n_field,3,3) to each row's self block; *missing counts rows
 * without one (device int). */
int mbem_near_add_diagonal(const int64_t* rowptr, const int64_t* cols, double* vals, int64_t n_field,
                           const double* D, int* missing, void* stream);
/* y = A x for the mixed operator (far in double-float, near in FP64);
 * y (n_rows) is overwritten. work >= 2 n_cols floats + 64 bytes.
 * The product streams the far field through a bulk-copy ring whose waits are
 * bounded: a wait that runs out sets a device flag and the product returns
 * MBEM_OK with a partial y. The flag is read (and cleared) only by
 * mbem_mixed_wait_check or by the next FGMRES solve on a mixed operator. */
int mbem_mixed_matvec(const mbem_mixed_operator* op, const double* x, double* y, void* work,
                      size_t work_bytes, void* stream);
/* MBEM_ERR_WAIT if a bulk-copy wait of a mixed-operator kernel (product or
 * assembly) gave up since the last check, else MBEM_OK; clears the flag.
 * Synchronises `stream`. No counterpart in the reference (its products
 * cannot time out). */
int mbem_mixed_wait_check(void* stream);
/* The same product for callers that cannot allocate device memory (a host that
 * gives all device memory to its own pool at start-up, or a loop that must not
 * enter the allocator): no workspace argument, and nothing allocated. Its
 * scratch is a fixed 2 MiB array inside the library, held by every GPU that
 * loads it until exit, so n_cols is limited to 262144 (larger sizes return
 * MBEM_ERR_SIZE). The first call on each device looks the array's device
 * address up (cudaGetSymbolAddress) and must come before any stream capture;
 * the address is cached per CUDA context, so after cudaDeviceReset the first
 * call in the new context again comes before any capture.
 * All calls share the array: calls that overlap on the GPU (other streams,
 * other host threads) race and must be serialised by the caller.
 * An expired bulk-copy wait is reported as for mbem_mixed_matvec: run
 * mbem_mixed_wait_check after the product to see it.
 * It has no counterpart in the reference. */
int mbem_mixed_matvec_noalloc(const mbem_mixed_operator* op, const double* x, double* y,
                              void* stream);

/* ---- BF16 inner operator and inner solve (the mixed-precision
 * preconditioner). A16 is the mixed operator's FP32 far field rounded to
 * BF16 (round to nearest even; BF16 keeps FP32's exponent range, so no block
 * scales are needed); the near blocks stay FP64.
 * y = A16 x + near blocks x, FP32 row sums; work: n_cols floats. */
int mbem_bf16_matvec(const uint16_t* A16, int64_t ld16, int64_t n_rows, int64_t n_cols, int n_near,
                     const mbem_near_blocks* near, const double* x, double* y, void* work, size_t work_bytes,
                     void* stream);

/* z = the iterate after `iterations` steps of GMRES from zero on
 * P (A16 + near) P z = P r (P: the deflation of params->u_ranges), as a
 * flexible right preconditioner of FGMRES on the accurate operator: the inner
 * steps read 2 bytes per far entry, the outer ones 4. The Arnoldi steps, the
 * Givens rotations and the back substitution run on the device; the host
 * enqueues step j + 1 before it reads step j's small status block (pinned
 * memory behind an event), and stops enqueueing once a step ended the basis
 * (residual estimate below rtol |P r|, rtol > 0; an invariant Krylov space;
 * a zero pivot): the one step already queued behind it returns at once on
 * the device. It does not synchronise `stream`: z is ready in stream order. */
#define MBEM_INNER_MAX_ITERS 64
typedef struct {
    int64_t n;                      /* system size (square) */
    const uint16_t* A16;            /* (n, ld16) row-major BF16, 16-byte aligned */
    int64_t ld16;                   /* multiple of 8 */
    int n_near;
    const mbem_near_blocks* near;   /* HOST array of n_near FP64 near-block lists */
    int iterations;                 /* at most this many steps, 1..MBEM_INNER_MAX_ITERS */
    double rtol;                    /* > 0: stop once the inner residual estimate is below rtol |P r|;
                                       0: all steps (an exact breakdown still ends the basis) */
    int n_u_ranges;                 /* deflation ranges, as in mbem_fgmres_params */
    const int64_t* u_ranges;
    void* work;                     /* mbem_inner_bf16_workspace_size(n, iterations) bytes */
    size_t work_bytes;
    int precond;                    /* 0: none; 1: block-Jacobi, 2: learned two-level (as in
                                       mbem_fgmres_params), a fixed right preconditioner M of the
                                       inner GMRES: steps on A16 M, result z = P M (V y) */
    const void* precond_state;      /* mbem_block_jacobi* / mbem_nn_precond* (host pointer) */
} mbem_inner_bf16;
size_t mbem_inner_bf16_workspace_size(int64_t n, int iterations);
int mbem_inner_bf16_apply(const mbem_inner_bf16* p, const double* r, double* z, void* stream);
/* Inner steps, applications and (when timed) the device time of their BF16
 * products in ms since the last call; resets them and sets whether the
 * following applications time their products with CUDA events. */
void mbem_inner_bf16_stats(int timing, int64_t* steps, int64_t* applies, double* matvec_ms);

/* ---- dense LU with partial pivoting in FP32 (la/lu.py Factor with FP32
 * factors; the caller refines in FP64). In place on A (n x n at lda);
 * piv[k] = the row exchanged with row k at step k (0-based, LAPACK order);
 * *info (device int) = first zero pivot + 1, or 0. work: device memory of
 * mbem_lu_workspace_size(n, SM count) bytes. The panel runs as a cooperative
 * launch with bounded grid barriers (MBEM_ERR_WAIT if one runs out). */
size_t mbem_lu_workspace_size(int64_t n, int sms);
int mbem_lu_factor_f32(float* A, int64_t lda, int64_t n, int32_t* piv, void* work, size_t work_bytes, int* info,
                       void* stream);
/* x = A^-1 b from the factors (b, x FP64 device vectors; perm[i] = the
 * original row at position i after all interchanges; xf: n floats). */
/* X = A^-1 B for k right-hand sides (row-major FP64 n x k at ldb / ldx) from
 * the FP32 factors: blocked triangular solves with tensor-core updates
 * (FP32-accurate); work: mbem_lu_solve_many_workspace_size(n, k) bytes. */
size_t mbem_lu_solve_many_workspace_size(int64_t n, int64_t k);
int mbem_lu_solve_many_f32(const float* LU, int64_t lda, int64_t n, const int32_t* perm, const double* B,
                           int64_t ldb, int64_t k, double* X, int64_t ldx, void* work, size_t work_bytes,
                           void* stream);
/* Device ms of the factorisations' phases since the last call (phase_ms[3]:
 * the panels with their interchanges, the U block rows, the tensor-core
 * trailing updates); resets them and switches the phase timing of later
 * factorisations on or off. */
void mbem_lu_stats(int timing, double* phase_ms);
int mbem_lu_solve_f32(const float* LU, int64_t lda, int64_t n, const int32_t* perm, const double* b, double* x,
                      float* xf, void* stream);
/* x = A^-T b from the same factors (A^T = U^T L^T P): the second product of
 * the 1-norm condition estimator, which the reference takes from LAPACK's
 * gecon on its factors or onenormest on single-precision ones
 * (src/mbem/la/lu.py:241-258). */
int mbem_lu_solve_t_f32(const float* LU, int64_t lda, int64_t n, const int32_t* perm, const double* b, double* x,
                        float* xf, void* stream);

/* ---- tile configurations of the tunable kernel families (the autotuner's
 * knobs). Each family has mbem_tune_count() candidates; the choice is
 * process-wide (configuration 0 until set) and applies to the next launch. */
enum {
    MBEM_TUNE_MIXED_MATVEC = 0,   /* FP32 double-float matvec: rows x chunk x stages */
    MBEM_TUNE_BF16_MATVEC = 1,    /* BF16 inner matvec: rows x chunk x stages */
    MBEM_TUNE_MM_MATVEC = 2,      /* persistent multi-mesh matvec: chunk x stages */
    MBEM_TUNE_GEMM_SPLIT = 3,     /* tensor-core GEMM K split: cost model or fixed */
    MBEM_TUNE_FAMILIES = 4
};
int mbem_tune_count(int family);
int mbem_tune_get(int family);
int mbem_tune_set(int family, int config);
int mbem_tune_describe(int family, int config, char* buf, int len);

/* ---- many unevenly sized meshes in one solve. Each mesh keeps its mixed
 * operator (FP32 far field + FP64 near blocks by field point, the calibrated
 * diagonal inside them); the batch vectors hold the meshes' unknowns one
 * after another, each segment rounded up to MBEM_MM_SEGMENT entries (padding
 * zero). One persistent launch applies every mesh's operator; deflated
 * GMRES(restart) runs on all meshes in lockstep with per-mesh reductions and
 * Givens rotations on the device, each restart cycle one CUDA graph launch
 * (use_graph = 1) or the same kernels launched one by one (0). ---------- */
#define MBEM_MM_SEGMENT 512
#define MBEM_MM_MAX_RESTART 64
typedef struct {
    const float* A32;        /* (n, ld32) FP32 far field, 16-byte aligned, ld32 % 4 == 0 */
    int64_t ld32;
    int64_t n;               /* unknowns (a multiple of 3) */
    int64_t offset;          /* segment start: 0 for the first mesh, then the previous
                                offset + n rounded up to MBEM_MM_SEGMENT */
    const int64_t* rowptr;   /* near blocks by field point: (n/3 + 1) row pointers, */
    const int64_t* cols;     /* source node per block (columns 3c..3c+2), */
    const double* vals;      /* 3x3 FP64 values per block, row-major */
    int64_t u_off, u_len;    /* deflated u-slot range within the segment (u_len = 0: none) */
    const uint16_t* A16;     /* optional BF16 copy of the far field (n, ld16), 16-byte aligned,
                                ld16 % 8 == 0: the inner operator of mbem_mm_solve_mixed */
    int64_t ld16;
} mbem_mm_mesh;

typedef struct {
    int* iterations;         /* HOST arrays of n_mesh entries, filled by the solve */
    double* relres;          /* true relative residual at the last check */
    int* converged;
    int cycles;              /* restart cycles run */
} mbem_mm_report;

typedef struct mbem_mm_solver mbem_mm_solver;
/* batch vector length (-1 if the layout is invalid) and workspace bytes (0 if invalid) */
int64_t mbem_mm_total(const mbem_mm_mesh* meshes, int n_mesh);
size_t mbem_mm_workspace_size(const mbem_mm_mesh* meshes, int n_mesh, int restart);
/* work: device memory (256-byte aligned) that the solver keeps; the meshes'
 * arrays must outlive it. */
int mbem_mm_create(const mbem_mm_mesh* meshes, int n_mesh, int restart, void* work, size_t work_bytes,
                   void* stream, mbem_mm_solver** out);
void mbem_mm_destroy(mbem_mm_solver* solver);
/* y = A x on every mesh (batch vectors) */
int mbem_mm_matvec(mbem_mm_solver* solver, const double* x, double* y, void* stream);
/* x = the deflated solution of every mesh to rtol (true residual), at most
 * max_cycles restart cycles; graph capture needs a stream other than the
 * legacy default stream. */
int mbem_mm_solve(mbem_mm_solver* solver, const double* b, double* x, double rtol, int max_cycles, int use_graph,
                  mbem_mm_report* report, void* stream);
/* The mixed-precision batch solve: refinement on the accurate operator whose
 * corrections are lockstep GMRES solves on the BF16 far fields (every mesh's
 * A16) to inner_rtol of each residual; at most max_outer refinement steps and
 * max_cycles restart cycles an inner solve. report->iterations: inner steps;
 * report->cycles: refinement steps. */
int mbem_mm_solve_mixed(mbem_mm_solver* solver, const double* b, double* x, double rtol, double inner_rtol,
                        int max_outer, int max_cycles, int use_graph, mbem_mm_report* report, void* stream);
/* MBEM_ERR_WAIT if a bounded wait of the batched matvec gave up since the last check */
int mbem_mm_check(void* stream);

/* ---- cluster block-Jacobi preconditioner (la/preconditioner.py:421-470,
 * the "block_jacobi" rung; chunks from la/cluster.py:56-75 bisection, built
 * by the caller). The chunks partition 0..n-1; chunk c holds the DOFs
 * dofs[chunk_ptr[c] .. chunk_ptr[c+1]) (at most MBEM_BJ_MAX_DOF of them,
 * so that a chunk's FP32 copy fits one CTA's shared memory). local[d] is
 * the position of DOF d in its chunk and chunk_of[d] its chunk (both needed
 * by the mixed build only). inv holds mbem_bj_inverse_bytes() of FP32
 * inverses, written by a build, read by mbem_bj_apply. All device memory
 * is the caller's. --------------------------------------------------- */
#define MBEM_BJ_MAX_DOF 225
typedef struct {
    int64_t n;                  /* system size */
    int64_t n_chunks;
    int m_max;                  /* largest chunk (DOF), <= MBEM_BJ_MAX_DOF */
    const int64_t* chunk_ptr;   /* (n_chunks + 1) device */
    const int64_t* dofs;        /* (n) device */
    const int32_t* local;       /* (n) device */
    const int32_t* chunk_of;    /* (n) device */
    float* inv;                 /* (n_chunks, m_max, m_max) device */
} mbem_block_jacobi;

size_t mbem_bj_inverse_bytes(int64_t n_chunks, int m_max);
/* Inverts the diagonal chunks of a dense FP64 A (at ld) / of a mixed operator
 * (FP32 far field plus its FP64 near blocks). MBEM_ERR_NUMERIC when a chunk is
 * singular (its inverse is then the identity). */
int mbem_bj_build_dense(const double* A, int64_t ld, const mbem_block_jacobi* bj, void* stream);
int mbem_bj_build_mixed(const mbem_mixed_operator* op, const mbem_block_jacobi* bj, void* stream);
/* z = M^-1 r (r, z distinct device vectors of length n). */
int mbem_bj_apply(const mbem_block_jacobi* bj, const double* r, double* z, void* stream);

/* ---- learned preconditioner: block-Jacobi with a learned coarse space (no
 * reference counterpart: it replaces the block-Jacobi rung of
 * la/preconditioner.py:421-470 in the solve). Each block-Jacobi chunk c gets
 * six coarse vectors: its three translations and three learned vectors whose
 * 3x3 block on node i of the chunk is phi_i, the output of a small MLP on the
 * node's geometry; on node i the basis block is [I | phi_i] (3 x 6). With
 * Phi (n x 6C) and A_c = Phi^T A Phi:
 *     y = A_c^-1 Phi^T r,   z = Phi y + BJ (r - (A Phi) y).
 * MLP: MBEM_NN_FEAT -> MBEM_NN_HIDDEN (tanh) -> MBEM_NN_HIDDEN (tanh) -> 9
 * (phi_i row-major); flat FP32 parameters W1 (H x F), b1, W2 (H x H), b2,
 * W3 (9 x H), b3. Node i owns unknowns 3i..3i+2; every chunk holds whole
 * nodes. ---------------------------------------------------------------- */
#define MBEM_NN_FEAT 16
#define MBEM_NN_HIDDEN 32
#define MBEM_NN_PARAMS (MBEM_NN_HIDDEN * MBEM_NN_FEAT + MBEM_NN_HIDDEN + MBEM_NN_HIDDEN * MBEM_NN_HIDDEN + \
                        MBEM_NN_HIDDEN + 9 * MBEM_NN_HIDDEN + 9)
typedef struct {
    int64_t n;                       /* unknowns (a multiple of 3) */
    int64_t n_coarse;                /* 6 x the block-Jacobi chunks */
    const mbem_block_jacobi* bj;     /* chunks and their inverses (host pointer; chunk_of required) */
    const float* basis;              /* (n, 6) device: the coarse basis row of every unknown, Phi[d, 6 c(d) + k]
                                        (the [I | phi_i] blocks, orthonormalised per chunk) */
    const double* APhi;              /* (n, n_coarse) device: A Phi, written by mbem_nn_setup_dense */
    const double* Ac_inv;            /* (n_coarse, n_coarse) device: A_c^-1, written by the setup */
    double* work;                    /* mbem_nn_apply_workspace_size() bytes, device */
    const float* APhi32;             /* or (n, ld32) FP32 A Phi and (n_coarse, ld32) FP32 A_c^-1 (written by */
    const float* Ac_inv32;           /* mbem_nn_setup_mixed; APhi and Ac_inv NULL then) */
    int64_t ld32;                    /* their leading dimension: >= n_coarse, a multiple of 4 */
} mbem_nn_precond;

/* The learned preconditioner on the mixed operator: A Phi (FP32) from the
 * BF16 inner operator (its A16 far field and FP64 near blocks), A_c = Phi^T A
 * Phi (+ U U^T from `shift`, n_shift columns, for a calibrated system's
 * translation null space) and A_c^-1 by mbem_dense_inverse_f32. Requires
 * nn->APhi32 (n x ld32) and nn->Ac_inv32 (n_coarse x ld32); work: at least
 * mbem_dense_inverse_f32_workspace_size(n_coarse) bytes. Synchronises
 * `stream`. No counterpart in the reference. */
int mbem_nn_setup_mixed(const mbem_inner_bf16* inner, const mbem_nn_precond* nn, const double* shift, int n_shift,
                        void* work, size_t work_bytes, void* stream);
/* idx (n, k) int64: the k nearest of n points (n, 3) FP32 (centred), the
 * point itself first, by squared distance then index; k <= 16. The node
 * neighbourhoods of the learned preconditioner's features. No counterpart in
 * the reference. */
int mbem_knn(const float* points, int64_t n, int k, int64_t* idx, void* stream);
/* The same FP32 setup for a dense FP64 operator A (n x n at ld): A Phi with
 * FP32 products, A_c, A_c^-1 (FP32). Replaces mbem_nn_setup_dense's FP64
 * setup where a faster, preconditioner-accurate one serves. */
int mbem_nn_setup_dense32(const double* A, int64_t ld, const mbem_nn_precond* nn, const double* shift, int n_shift,
                          void* work, size_t work_bytes, void* stream);
/* M (n x n, row-major FP32 at ld >= n, device) = M^-1 in place. From n = 1024
 * a blocked Gauss-Jordan without row interchanges is tried first (64-column
 * blocks: the diagonal block inverted by one CTA, the rest updated on the
 * tensor cores with both factors in three BF16 pieces); it stands when no pivot was zero or non-finite and |A X v - v| <=
 * 1e-3 |v| for two fixed vectors v. Otherwise, and below n = 1024, Gauss-
 * Jordan with partial pivoting, 16 pivot columns a step (a one-CTA panel,
 * then one rank-16 update of the other columns); n <= 3214 (the panel lives
 * in shared memory). MBEM_ERR_NUMERIC when a column has no usable pivot.
 * Synchronises `stream`. No counterpart in the reference (it solves its small
 * systems with LAPACK on the host). */
size_t mbem_dense_inverse_f32_workspace_size(int64_t n);
int mbem_dense_inverse_f32(float* M, int64_t n, int64_t ld, void* work, size_t work_bytes, void* stream);
/* How many mbem_dense_inverse_f32 calls since the last call stood without
 * row interchanges, and how many ran the pivoted inverse; resets both. */
void mbem_dense_inverse_f32_stats(int64_t* no_interchange, int64_t* pivoted);
/* One level of the principal-axis bisection of points (m x 3 FP64, device)
 * that makes the block-Jacobi chunks (src/mbem/la/cluster.py:56-75, as
 * build_cluster_tree splits; the reference runs it on the host with numpy).
 * Segment s is order[seg_start[s] .. + seg_size[s]); a segment of at most
 * max_nodes points is a leaf. mbem_cluster_stats writes mean (n_seg x 3) and
 * stats (n_seg x 10: the count, then the 3 x 3 sums of (p - mean)(p -
 * mean)^T) of every non-leaf segment; the caller finds each leading
 * eigenvector (axis, n_seg x 3). mbem_cluster_split writes order_out: every
 * non-leaf segment partitioned stably into its points with a projection on
 * the axis below the median (the mean of the two middle order statistics)
 * and the rest, nl[s] = the left count; a segment with an empty side is
 * copied unchanged with nl[s] = -1, the projections (proj, m) left for the
 * caller's rank rule; a leaf is copied with nl[s] = its size. */
int mbem_cluster_stats(const double* pts, const int64_t* order, const int64_t* seg_start, const int64_t* seg_size,
                       int64_t n_seg, int max_nodes, double* mean, double* stats, void* stream);
int mbem_cluster_split(const double* pts, const int64_t* order, int64_t* order_out, const int64_t* seg_start,
                       const int64_t* seg_size, int64_t n_seg, int max_nodes, const double* mean, const double* axis,
                       double* proj, int64_t* nl, void* stream);
/* out (n_items, 9) = MLP(feat (n_items, MBEM_NN_FEAT)); act (n_items, 2H)
 * keeps the hidden activations for training (NULL at inference). */
int mbem_nn_forward(const float* feat, int64_t n_items, const float* params, float* act, float* out,
                    void* stream);
/* Training loss: the chunk-wise least-squares projection error (normal
 * equations regularised by 1e-8 trace / 6) of the block-Jacobi errors eps
 * (n_samples, n) onto each chunk's six coarse vectors, weighted by
 * inv_e2 (1/|eps_s|^2) and averaged, into *loss (device double); dphi
 * (n/3, 9) = dloss/dphi. partial: bj->n_chunks device doubles. */
int mbem_nn_coarse_loss_grad(const mbem_block_jacobi* bj, const float* phi, const float* eps,
                             const float* inv_e2, int64_t n_samples, float* dphi, double* partial,
                             double* loss, void* stream);
/* grad (MBEM_NN_PARAMS) = dloss/dparams from dloss/dout (n_items, 9). */
size_t mbem_nn_backward_workspace_size(int64_t n_items);
int mbem_nn_backward(const float* feat, int64_t n_items, const float* params, const float* act, const float* G,
                     float* grad, void* work, size_t work_bytes, void* stream);
/* One Adam step (step >= 1) on n parameters. */
int mbem_nn_adam(float* params, const float* grad, float* m, float* v, int64_t n, float lr, float beta1,
                 float beta2, float eps, int step, void* stream);
/* basis (n, 6) FP32: every chunk's [I | phi_i] rows orthonormalised (the
 * span is what the coarse correction depends on; an orthonormal basis keeps
 * A_c as well conditioned as A), and U (n_coarse, 3) = basis^T Z for the
 * rigid translations Z of the u-ranges (U may be NULL; with no u-range it
 * is left untouched). */
int mbem_nn_basis(const mbem_block_jacobi* bj, const float* phi, const int64_t* u_ranges, int n_u_ranges,
                  float* basis, double* U, void* stream);
/* A Phi, A_c and A_c^-1 (Gauss-Jordan, partial pivoting) for a dense FP64 A.
 * shift (n_coarse, n_shift) device, or NULL: A_c += shift shift^T first, with
 * shift = Phi^T Z for a calibrated operator whose null space Z (the rigid
 * translations of the u-slots, A Z = 0) the coarse space contains; the
 * solution on the complement of Z is unchanged. MBEM_ERR_NUMERIC when A_c is
 * singular. */
size_t mbem_nn_setup_workspace_size(int64_t n_coarse);
/* The two halves of the setup: A Phi and A_c (+ shift shift^T) into
 * APhi / Ac_inv, then A_c inverted in place. */
int mbem_nn_coarse_operator_dense(const double* A, int64_t ld, const mbem_nn_precond* nn, const double* shift,
                                  int n_shift, void* stream);
/* In-place inverse of a dense FP64 matrix (n x n, row-major, n <= 1,048,560)
 * by Gauss-Jordan with partial pivoting, one launch per pivot;
 * MBEM_ERR_NUMERIC when singular. */
size_t mbem_dense_inverse_workspace_size(int64_t n);
int mbem_dense_inverse(double* M, int64_t n, void* work, size_t work_bytes, void* stream);
int mbem_nn_setup_dense(const double* A, int64_t ld, const mbem_nn_precond* nn, const double* shift,
                        int n_shift, void* work, size_t work_bytes, void* stream);
/* z = M^-1 r (r, z distinct device vectors of length n). */
size_t mbem_nn_apply_workspace_size(int64_t n, int64_t n_coarse);
int mbem_nn_apply(const mbem_nn_precond* nn, const double* r, double* z, void* stream);

/* ---- many right-hand sides on the tensor cores: Y (M x n_rhs, FP32, at ldy)
 * = A (M x K, BF16 row-major at lda) X, with X passed transposed as Xt
 * (n_rhs x K, BF16 row-major at ldx), n_rhs <= 256; tcgen05.mma with TMA
 * operand staging and FP32 accumulation in tensor memory. The product of
 * the multi-RHS refinement (la/lu.py:210) and of batched FGMRES. lda and ldx
 * multiples of 8, bases 16-byte aligned. mbem_gemm_bf16_check synchronises
 * the stream and returns MBEM_ERR_WAIT if a pipeline wait of an earlier GEMM
 * gave up. --------------------------------------------------------------- */
int mbem_gemm_bf16(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K, int n_rhs,
                   float* Y, int64_t ldy, void* stream);
/* The same product written transposed: Yt (n_rhs x M) at ldy, one row per
 * right-hand side (the layout of the batched solver's vectors). */
int mbem_gemm_bf16_t(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K, int n_rhs,
                     float* Yt, int64_t ldy, void* stream);
/* The transposed product with K split over the SMs (up to 8 slices whose
 * partial sums are added in slice order): for products whose 128-row tiles
 * do not fill the GPU evenly. work: mbem_gemm_bf16_workspace_size() bytes. */
size_t mbem_gemm_bf16_workspace_size(int64_t M, int n_rhs);
int mbem_gemm_bf16_t_split(const void* A, int64_t lda, const void* Xt, int64_t ldx, int64_t M, int64_t K,
                           int n_rhs, float* Yt, int64_t ldy, void* work, size_t work_bytes, void* stream);
int mbem_gemm_bf16_check(void* stream);
/* C[M x N] -= A[M x K] Bt[N x K]^T on the tensor cores (BF16 row-major
 * operands, lda and ldb multiples of 8; FP32 C at ldc): the update of the
 * blocked LU and its solves. */
int mbem_gemm_bf16_sub(const void* A, int64_t lda, const void* Bt, int64_t ldb, int64_t M, int64_t N, int64_t K,
                       float* C, int64_t ldc, void* stream);

/* ---- batched GMRES for a block of k right-hand sides (k Krylov iterations
 * sharing one GEMM per step; la/solver.py:115-245 per right-hand side).
 * Vectors are RHS-major (k, n) row-major; a Krylov basis V is (n_vec, k, n)
 * FP32; Hessenberg columns H are (n_vec, k) FP64. ----------------------- */
/* BF16 copy out (rows x cols at ldo) of an FP32 (is_f64 = 0) or FP64 matrix,
 * and of a mixed operator (FP32 far field plus its near blocks). */
int mbem_to_bf16(const void* A, int is_f64, int64_t lda, int64_t rows, int64_t cols, uint16_t* out, int64_t ldo,
                 void* stream);
int mbem_mixed_to_bf16(const mbem_mixed_operator* op, uint16_t* out, int64_t ldo, void* stream);
/* The two-part split A = hi + lo (hi = bf16(A), lo = bf16(A - hi); about
 * 2^-16 relative) of an FP32/FP64 matrix or of a mixed operator (lo may be
 * NULL there: hi alone). */
int mbem_to_bf16x2(const void* A, int is_f64, int64_t lda, int64_t rows, int64_t cols, uint16_t* hi, uint16_t* lo,
                   int64_t ldo, void* stream);
int mbem_mixed_to_bf16x2(const mbem_mixed_operator* op, uint16_t* hi, uint16_t* lo, int64_t ldo, void* stream);
/* H[i, r] = V[i, r] . W[r] */
int mbem_batch_dots(const float* V, int n_vec, const float* W, int64_t k, int64_t n, double* H, void* stream);
/* W[r] += alpha sum_i H[i, r] V[i, r] */
int mbem_batch_axpy(float* W, const float* V, int n_vec, const double* H, double alpha, int64_t k, int64_t n,
                    void* stream);
/* norms[r] = |W[r]|, V[r] = W[r] / norms[r], Vbf (NULL or (k, n) BF16) its copy; W FP32 or FP64 */
int mbem_batch_normalize(const void* W, int w_is_f64, int64_t k, int64_t n, double* norms, float* V, uint16_t* Vbf,
                         void* stream);
/* X[r] += sum_i Y[i, r] V[i, r] (X FP64) */
int mbem_batch_update(double* X, const float* V, int n_vec, const double* Y, int64_t k, int64_t n, void* stream);
/* X[r] = P X[r]: the rigid translations of the u-ranges removed (FP32 or FP64 X) */
int mbem_batch_project(void* X, int is_f64, int64_t k, int64_t n, const int64_t* u_ranges, int n_u_ranges,
                       void* stream);
/* R = B - A X for the mixed operator and k right-hand sides (k, n) FP64: the
 * far field with FP32 entries and double-float accumulation, the near blocks
 * in FP64. */
size_t mbem_batch_residual_workspace_size(int64_t k, int64_t n);
int mbem_batch_residual_mixed(const mbem_mixed_operator* op, const double* B, const double* X, int64_t k, double* R,
                              void* work, size_t work_bytes, void* stream);

/* ---- mixed-precision stress readout of a nodal slip density (the elastic
 * stress, DD minus the exact eigenstress: evaluate.py:383-407 with
 * subtract_anelastic, tri_nodal.py:1131-1172): far pairs by FP32 quadrature
 * of the mollified point kernel (3x3, 5x5, 8x8 collapsed Gauss rules for
 * D / L above 12, above 6, below), near pairs (D <= near_factor max(eps, L))
 * by the FP64 nodal machinery. Two calls: prepare writes the per-source
 * records (mbem_readout_record_bytes), the per-observer near counts (n_obs)
 * and their scan rowptr (n_obs + 1), and returns the number of near pairs in
 * *n_near (host); evaluate takes near-pair buffers of that size (pair_obs
 * int64, pair_src int32, pair_out 9 doubles each) and writes out (n_obs, 3, 3)
 * (+)= alpha * stress. ------------------------------------------------- */
size_t mbem_readout_record_bytes(int64_t n_src);
int mbem_readout_prepare(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                         const double* eps, int64_t n_src, const double* density, int order, double near_factor,
                         float* records, int64_t* counts, int64_t* rowptr, int64_t* n_near, void* stream);
int mbem_readout_evaluate(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                          const double* eps, int64_t n_src, const double* density, double mu, double lam, int order,
                          const float* records, const int64_t* rowptr, int64_t n_near, int64_t* pair_obs,
                          int32_t* pair_src, double* pair_out, double alpha, int accumulate, double* out,
                          void* stream);
/* As mbem_readout_evaluate, and with eig_out (n_obs, 3, 3) also the
 * eigenstress of the same pairs (+)= alpha (evaluate_stress(parts=True)):
 * far pairs from the same quadrature points, near pairs by the FP64 nodal
 * closed form into pair_eig (9 doubles a near pair). eig_out NULL: the
 * elastic stress alone. */
int mbem_readout_evaluate_parts(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                                const double* eps, int64_t n_src, const double* density, double mu, double lam,
                                int order, const float* records, const int64_t* rowptr, int64_t n_near,
                                int64_t* pair_obs, int32_t* pair_src, double* pair_out, double* pair_eig,
                                double alpha, int accumulate, double* out, double* eig_out, void* stream);

/* ---- deflated FGMRES on a dense operator (la/solver.py:115-245 fgmres,
 * wired as backends/hmat.py:678-690: P A P y = P b, P = I - Z Z^T with Z
 * the rigid-translation basis of backends/dense.py:190-208). ---------- */
typedef struct {
    int restart;            /* Krylov dimension per cycle (la/solver.py restart) */
    int maxiter;            /* total iteration cap */
    double rtol;            /* relative residual target on the true residual */
    int stagnation_window;  /* iterations without a stagnation_factor gain before stopping */
    double stagnation_factor;
    int n_u_ranges;         /* deflation: number of (offset, size) u-slot ranges, 0 = none */
    const int64_t* u_ranges;/* HOST array of 2*n_u_ranges int64 */
    int precond;            /* 0 none, 1 block-Jacobi (state: const mbem_block_jacobi*),
                               2 learned (state: const mbem_nn_precond*),
                               3 BF16 inner solve (state: const mbem_inner_bf16*) */
    const void* precond_state; /* the preconditioner object for precond != 0 (host pointer) */
    int time_matvec;        /* 1: time every operator application with CUDA events */
    int x_is_zero;          /* 1: x is zero on entry (skips the first product); 0: x is the initial guess */
} mbem_fgmres_params;

typedef struct {
    int converged;
    int iterations;
    int restarts;
    int stagnated;
    double true_relres;
    double arnoldi_relres;
    double* history;        /* optional HOST array of maxiter doubles, filled if non-NULL */
    int matvecs;            /* operator applications (A x products) */
    double matvec_ms;       /* their total device time when params->time_matvec */
} mbem_fgmres_report;

/* Bytes of device workspace mbem_fgmres_dense / mbem_fgmres_mixed need for
 * n unknowns. */
size_t mbem_fgmres_workspace_size(int64_t n, int restart);

/* As mbem_fgmres_dense for the mixed operator: the residuals and the true
 * residual are those of the mixed operator, evaluated to ~1e-14. */
int mbem_fgmres_mixed(const mbem_mixed_operator* op, const double* b, double* x,
                      const mbem_fgmres_params* params, void* work, size_t work_bytes,
                      mbem_fgmres_report* report, void* stream);

/* Solve A x = b (A FP64 (n,n) at leading dimension ld; b, x device (n,)).
 * x holds the initial guess on entry (zeros for none) and the solution on
 * exit (the zero-mean-translation representative P y when deflating).
 * The Gram-Schmidt passes, |w| and the Givens rotation of each step run on
 * the device; the host waits for each step's small status block (an event,
 * not a stream-wide wait) for its stopping and stagnation tests, and the
 * call synchronises `stream` once at its end. */
int mbem_fgmres_dense(const double* A, int64_t ld, int64_t n, const double* b, double* x,
                      const mbem_fgmres_params* params, void* work, size_t work_bytes,
                      mbem_fgmres_report* report, void* stream);

/* The deflation projection v_out = P v_in (hmat.py:684-685 proj); v_out may
 * alias v_in. work: 384 doubles of device memory (partial sums). */
int mbem_project_translation(const double* v_in, double* v_out, int64_t n,
                             const int64_t* u_ranges, int n_u_ranges, double* work,
                             void* stream);

/* Mixed-precision displacement of a P0 slip density at many observers
 * (tri_nodal.py:1310-1319 t_disp_contract at order 0; evaluate.py:194-250):
 * out[f] (+)= alpha sum_s T(x_f, s) d_s. Far pairs by the FP32 quadrature of
 * the mixed operator's far field, near pairs (centroid distance below
 * near_factor max(eps, h) or 1.5 L) by the FP64 closed form. coeffs: the six
 * t_coeffs (host). Within ~1e-6 of the FP64 contraction. */
int mbem_t_disp_readout(const double* x, int64_t n_obs, const double* tri_verts, const double* normals,
                        const double* eps, int64_t n_src, const double* density, const double* coeffs,
                        double near_factor, double alpha, int accumulate, double* out, void* stream);

/* ---- Mesh geometry for a batch of points (the volume sampler) -----------
 * Replaces src/mbem/geometry.py:8-57 (solid_angle_batch, the
 * _solid_angle_rows kernel behind RegionModel.point_in_region,
 * src/mbem/model/core.py:994-1025) and src/mbem/geometry.py:60-105
 * (point_triangle_distance, distance_to_mesh). tri_verts: (n_tri, 3, 3)
 * FP64; points: (n_pts, 3) FP64; records: mbem_geom_record_bytes(n_tri)
 * bytes of 16-byte aligned device memory that mbem_geom_prepare fills once
 * per mesh. Far pairs run in FP32 on hi/lo split coordinates, near pairs
 * (within 4 circumradii) in FP64; the solid-angle sum is within ~1e-6 sr
 * of the FP64 sum. ------------------------------------------------------ */
size_t mbem_geom_record_bytes(int64_t n_tri);
int mbem_geom_prepare(const double* tri_verts, int64_t n_tri, float* records, void* stream);
/* total[i] (+)= weight * sum_t Omega_t(points[i]) (accumulate 0: =). */
int mbem_solid_angle_sum(const float* records, const double* tri_verts, int64_t n_tri, const double* points,
                         int64_t n_pts, double weight, int accumulate, double* total, void* stream);
/* dist[i], idx[i]: the exact distance from points[i] to the nearest triangle
 * and its index, over every triangle of the mesh (ties: nearer centroid,
 * then lower index). max_edge: the mesh's longest edge (sets the FP32
 * candidate margin). n_tri >= 1. */
int mbem_mesh_distance(const float* records, const double* tri_verts, int64_t n_tri, const double* points,
                       int64_t n_pts, double max_edge, double* dist, int64_t* idx, void* stream);

/* ---- compressed pair operator: one (field mesh, source mesh, kernel) pair
 * with P0 sources, its admissible blocks in low-rank form and the rest
 * dense (src/mbem/la/hop.py:137 PairCompressed, :489 matvec; la/aca.py
 * compress_block / aca_single; la/flatview.py FlatView). Elements are
 * numbered in the cluster-tree order, so that every block is a pair of
 * contiguous element ranges; the caller keeps the permutation. Factors and
 * dense blocks are stored in FP32 (the reference's storage type at a block
 * tolerance >= 1e-5, flatview.py:127-136). ------------------------------ */
typedef struct {
    int kernel;                /* 0 T ("H", 6 coefficients), 1 U ("G", 3) */
    const double* x_field;     /* (n_field, 3) collocation points, tree order, device */
    int64_t n_field;
    const double* tri_verts;   /* (n_src, 9) source corners, tree order, device */
    const double* normals;     /* (n_src, 3) source normals (T kernel), device */
    const double* eps;         /* (n_src) mollifier radii, device */
    int64_t n_src;
    double coeffs[6];          /* basis.py t_coeffs / u_coeffs of the material */
    double near_factor;        /* pairs within near_factor * max(eps, mean edge) or 1.5 longest edges
                                  of the source centroid take the FP64 closed form, the rest the FP32
                                  far quadrature (the mixed operator's split) */
    void* prep;                /* device, mbem_pair_prep_bytes; filled by mbem_pair_prepare */
} mbem_pair_geometry;
size_t mbem_pair_prep_bytes(int64_t n_field, int64_t n_src);
int mbem_pair_prepare(const mbem_pair_geometry* g, void* stream);

/* Cross approximation of a batch of admissible blocks (aca.py:334-419
 * aca_single, :579-658 compress_block): one CTA per block, 3 x 3 element
 * pivots, stopped when the residual on 10 x 10 sampled element pairs falls
 * below tol / 2 of the sample's norm; certified on 3 random element rows and
 * 3 random element columns evaluated exactly; a certificate above 3 tol
 * reruns the block at tol / 10 and a second failure, or the rank cap,
 * leaves the block to be applied exactly. Factors are written transposed:
 * U^T (3 max_pivots[i] rows of pad4(3 nr[i]) floats) at U + u_off[i] and
 * V^T likewise at V + v_off[i] (offsets multiples of 4 floats). */
#define MBEM_ACA_LOWRANK 0
#define MBEM_ACA_CAPPED 1       /* the rank cap was reached: apply exactly */
#define MBEM_ACA_FAILED 2       /* the retry failed its certificate too: apply exactly */
#define MBEM_ACA_RETRIED 4      /* flag: the first certificate failed */
typedef struct {
    int64_t n_blocks;
    const int32_t* r0;          /* device (n_blocks): first field element of each block */
    const int32_t* nr;          /*   field elements */
    const int32_t* c0;          /*   first source element */
    const int32_t* nc;          /*   source elements */
    const int32_t* max_pivots;  /*   rank cap in element pivots (aca.py:618-620) */
    const int64_t* u_off;       /*   float offsets of each block's factors */
    const int64_t* v_off;
    float* U;
    float* V;
    int32_t* rank;              /* out: factor columns, 3 x pivots (0 unless low rank) */
    int32_t* status;            /* out: MBEM_ACA_* */
    float* err;                 /* out: certified relative Frobenius error of the factors kept */
    double tol;                 /* block tolerance (BLOCK_COMPRESSION_TOL) */
    uint64_t seed;              /* sample and certificate lines of block i come from (seed, first_index + i) */
    int64_t first_index;
    int max_nr, max_nc, max_pivots_all;  /* maxima over the batch (shared-memory size) */
} mbem_aca_batch;
int mbem_aca_compress(const mbem_pair_geometry* g, const mbem_aca_batch* b, void* stream);
/* Recompression of cross-approximation factors (aca.py:422-438 recompress):
 * the SVD of U V^T truncated at tol / 2, through its K x K core (double-float
 * Grams, FP64 Cholesky factors Ru, Rv, one-sided Jacobi on C = Ru Rv^T in
 * FP32; U' = U Rv^T Y_k, V' = V Ru^T (C Y)_k S_k^-2), written transposed to
 * Ur / Vr (capacity rank[i] rows each) and certified on the block's
 * certificate lines (those of mbem_aca_compress for the same seed and block
 * index); rank_out[i] = the columns kept, or 0 when the block is not
 * recompressed (rank outside [2, max_rank]) or its certificate exceeds 3 tol. */
typedef struct {
    int64_t n_blocks;
    const int32_t* r0;
    const int32_t* nr;
    const int32_t* c0;
    const int32_t* nc;
    const int32_t* rank;        /* factor columns of the cross approximation */
    const int64_t* u_off;       /* its factors, as mbem_aca_compress wrote them */
    const int64_t* v_off;
    const float* U;
    const float* V;
    const int64_t* ur_off;      /* out: float offsets of the recompressed factors */
    const int64_t* vr_off;
    float* Ur;
    float* Vr;
    int32_t* rank_out;
    float* err_out;
    const int64_t* index;       /* the block's index for its certificate lines */
    double tol;
    uint64_t seed;
    int max_rank;               /* at most 64 (shared-memory size) */
} mbem_aca_recompression;
int mbem_aca_recompress(const mbem_pair_geometry* g, const mbem_aca_recompression* r, void* stream);
/* Copies the first rank[i] rows of each block's U^T and V^T from the batch
 * scratch to their final offsets. */
int mbem_aca_compact(int64_t n_blocks, const int32_t* nr, const int32_t* nc, const int32_t* rank,
                     const int64_t* u_src, const int64_t* v_src, const float* U_src, const float* V_src,
                     const int64_t* u_dst, const int64_t* v_dst, float* U_dst, float* V_dst, void* stream);
/* Dense blocks (flatview.py:41-118 dense_leaves): block i transposed, D^T as
 * 3 nc rows of pad4(3 nr) FP32 (padding zero), at D + d_off[i]; col_ptr
 * (n_blocks + 1) is the prefix sum of nc (one thread per block column). */
int mbem_pair_dense_blocks(const mbem_pair_geometry* g, int64_t n_blocks, const int32_t* r0, const int32_t* nr,
                           const int32_t* c0, const int32_t* nc, const int64_t* d_off, const int64_t* col_ptr,
                           float* D, void* stream);

/* The flat operator of one material (FlatView): low-rank blocks, dense
 * blocks, and the field rows cut into strips (the finest ranges every block's
 * rows are a union of); strip s owns rows [strip_r0, strip_r0 + strip_nr)
 * (elements) and applies the blocks strip_items[strip_ptr[s] ..
 * strip_ptr[s+1]) in that order (id < n_lr: low rank; else n_lr + dense id),
 * so every output row has one writer and a fixed summation order. The
 * product streams each strip's blocks as units of MBEM_COMPRESSED_UNIT
 * factor rows: unit u = rows [unit_k0[u], unit_k0[u] + 32) of block
 * unit_item[u] (the transposed factor U^T, or D^T of a dense block), listed
 * per strip in item order at unit_ptr[s] .. unit_ptr[s+1]. */
#define MBEM_COMPRESSED_UNIT 32
typedef struct {
    int64_t n_field, n_src;       /* elements */
    const int64_t* field_order;   /* device: tree position -> field element */
    const int64_t* src_order;     /* device: tree position -> source element */
    int64_t n_lr;
    const int32_t* lr_r0;
    const int32_t* lr_nr;
    const int32_t* lr_c0;
    const int32_t* lr_nc;
    const int32_t* lr_rank;       /* factor columns */
    const int64_t* lr_u;          /* float offsets of U^T / V^T (rank rows of pad4(3 n) floats) */
    const int64_t* lr_v;
    const int64_t* lr_w;          /* offsets into the rank-sized projections (sum of ranks) */
    const float* U;
    const float* V;
    int64_t n_w;
    int64_t n_dense;
    const int32_t* d_r0;
    const int32_t* d_nr;
    const int32_t* d_c0;
    const int32_t* d_nc;
    const int64_t* d_off;
    const float* D;
    int64_t n_strips;
    const int32_t* strip_r0;
    const int32_t* strip_nr;
    const int64_t* strip_ptr;
    const int32_t* strip_items;
    int max_strip;                /* largest strip_nr */
    int max_lr_nc;                /* largest lr_nc */
    const int64_t* unit_ptr;      /* (n_strips + 1) */
    const int32_t* unit_item;
    const int32_t* unit_k0;
    int64_t n_proj;               /* the projections w_i = V_i^T x in units of four factor rows: */
    const int32_t* proj_block;    /*   unit u = rows proj_k0[u] .. +3 of low-rank block proj_block[u] */
    const int32_t* proj_k0;
} mbem_compressed_view;
size_t mbem_compressed_matvec_workspace_size(const mbem_compressed_view* v);
/* y (3 n_field, original element order) = A x (3 n_src); FP32 factors and
 * blocks, FP32 products summed per block, FP64 across blocks. */
int mbem_compressed_matvec(const mbem_compressed_view* v, const double* x, double* y, void* work,
                           size_t work_bytes, void* stream);
/* The operator as a dense FP64 (3 n_field, 3 n_src) matrix at ld (original
 * order), for checks at small sizes (FlatView.to_dense). */
int mbem_compressed_to_dense(const mbem_compressed_view* v, double* out, int64_t ld, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MBEM_GB300_H */
