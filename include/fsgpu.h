/*
 * fsgpu.h -- C ABI of the GB300-native Krylov backend (libfsgpu.so).
 *
 * The library is the device replacement for flecsolve's Krylov hot path:
 * the vector Data/Operations policy (flecsolve/vectors/core.hh:26-353,
 * vectors/operations/topo_view.hh:26-291), the CSR operator
 * (flecsolve/matrices/seq.hh:35-63, 177-193; matrices/parcsr.hh:29-177) and the
 * CG / BiCGSTAB / GMRES loops (flecsolve/solvers/cg.hh:43-139,
 * bicgstab.hh:39-187, gmres.hh:54-348).  Signatures use plain pointers, sizes
 * and opaque handles only.
 *
 * Conventions
 *  - Every call returns an int status (FS_OK = 0).  Nothing aborts; the
 *    message of the last failure on a context is fs_last_error().
 *  - One fs_ctx = one CUDA device + one CUDA stream.  Calls on a context are
 *    not thread-safe; different contexts may be driven from different threads.
 *  - Whoever creates a handle destroys it (fs_*_destroy).  Matrix and vector
 *    creation copies host data into library-owned device memory.
 *  - Reductions return their value through a host pointer and synchronise the
 *    context stream, which is the `.get()` of the reference's futures
 *    (flecsolve/util/future.hh:23-59).
 */
#ifndef FSGPU_H
#define FSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FS_API __attribute__((visibility("default")))
#else
#define FS_API
#endif

/* ------------------------------------------------------------ status --- */
enum fs_status {
	FS_OK = 0,
	FS_ERR_BAD_HANDLE = 1,     /* NULL or destroyed handle                  */
	FS_ERR_SIZE_MISMATCH = 2,  /* vector / matrix sizes disagree            */
	FS_ERR_OUT_OF_MEMORY = 3,  /* device allocation failed                  */
	FS_ERR_CUDA = 4,           /* a CUDA runtime call failed                */
	FS_ERR_NON_FINITE = 5,     /* NaN / Inf met where a finite value is due */
	FS_ERR_BREAKDOWN = 6,      /* a solver hit a reference flog_assert      */
	FS_ERR_INVALID_ARG = 7,    /* argument out of range                     */
	FS_ERR_NO_DEVICE = 8,      /* no usable CUDA device                     */
	FS_ERR_UNSUPPORTED = 9,    /* valid request the library does not handle */
	FS_ERR_IO = 10,            /* file missing, unreadable or malformed     */
	FS_ERR_CALLBACK = 11       /* a caller's operator callback failed       */
};

/* value types of vectors and matrix values */
enum fs_dtype { FS_F64 = 0, FS_F32 = 1 };

/* solve_info::stop_reason, flecsolve/solvers/solver_settings.hh:64-72 */
enum fs_stop_reason {
	FS_CONVERGED_ATOL = 0,
	FS_CONVERGED_RTOL = 1,
	FS_CONVERGED_USER = 2,
	FS_DIVERGED_DTOL = 3,
	FS_DIVERGED_ITERS = 4,
	FS_DIVERGED_BREAKDOWN = 5,
	FS_STATUS_UNKNOWN = 6
};

typedef struct fs_ctx_s *fs_ctx;
typedef struct fs_vec_s *fs_vec;
typedef struct fs_csr_s *fs_csr;
typedef struct fs_solver_s *fs_solver;
typedef struct fs_mm_s *fs_mm;
typedef struct fs_nka_s *fs_nka;
typedef struct fs_parcsr_s *fs_parcsr;

/* ----------------------------------------------------------- context --- */
/* Replaces the FleCSI runtime/scheduler context the reference's vector ops
 * run in (flecsolve/vectors/operations/topo_view.hh:38-40). */
FS_API int fs_ctx_create(int device, fs_ctx *out);
FS_API int fs_ctx_destroy(fs_ctx ctx);
FS_API int fs_ctx_sync(fs_ctx ctx);
/* the context's CUDA stream (a cudaStream_t) for interop */
FS_API int fs_ctx_stream(fs_ctx ctx, void **stream);
/* number of SMs of the context device */
FS_API int fs_ctx_sm_count(fs_ctx ctx, int *sms);
FS_API const char *fs_last_error(fs_ctx ctx);
FS_API const char *fs_status_string(int status);
/* number of kernels this library has launched on the context */
FS_API int fs_ctx_launch_count(fs_ctx ctx, int64_t *count);
/* CUDA-event timing on the context stream: record event `slot` (0..15) and
 * read the time between two recorded slots (synchronises on the later one) */
FS_API int fs_ctx_event_record(fs_ctx ctx, int slot);
FS_API int fs_ctx_event_elapsed(fs_ctx ctx, int slot_from, int slot_to, float *ms);

/* ----------------------------------------------------------- vectors --- */
/* Device Data policy: replaces vec::data::topo_view storage
 * (flecsolve/vectors/data/topo_view.hh:23-71) and seq_data
 * (flecsolve/vectors/seq.hh:40-67). */
FS_API int fs_vec_create(fs_ctx ctx, int64_t n, int dtype, fs_vec *out);
/* wrap caller-owned device memory (not freed by fs_vec_destroy) */
FS_API int fs_vec_wrap(fs_ctx ctx, int64_t n, int dtype, void *dptr, fs_vec *out);
FS_API int fs_vec_destroy(fs_vec v);
FS_API int fs_vec_size(fs_vec v, int64_t *n);
FS_API int fs_vec_dtype(fs_vec v, int *dtype);
FS_API int fs_vec_device_ptr(fs_vec v, void **dptr);
/* host <-> device copies of the whole vector (host data of the vector's dtype) */
FS_API int fs_vec_upload(fs_vec v, const void *host, int64_t n);
FS_API int fs_vec_download(fs_vec v, void *host, int64_t n);

/* Operations policy, flecsolve/vectors/core.hh:59-310 (argument meaning of the
 * reference: the last vector argument is `this`).  Aliasing of inputs and
 * output is allowed wherever the reference allows it
 * (operations/topo_view.hh:78-210). */
FS_API int fs_vec_copy(fs_vec src, fs_vec dst);                       /* core.hh:59  */
FS_API int fs_vec_zero(fs_vec x);                                     /* core.hh:67  */
FS_API int fs_vec_set_scalar(fs_vec x, double val);                   /* core.hh:75  */
FS_API int fs_vec_scale(double alpha, fs_vec x, fs_vec y);            /* y = alpha x, core.hh:84 */
FS_API int fs_vec_scale_self(double alpha, fs_vec x);                 /* core.hh:95  */
FS_API int fs_vec_add(fs_vec x, fs_vec y, fs_vec z);                  /* z = x + y   */
FS_API int fs_vec_subtract(fs_vec x, fs_vec y, fs_vec z);             /* z = x - y   */
FS_API int fs_vec_multiply(fs_vec x, fs_vec y, fs_vec z);             /* z = x * y   */
FS_API int fs_vec_divide(fs_vec x, fs_vec y, fs_vec z);               /* z = x / y   */
FS_API int fs_vec_reciprocal(fs_vec x, fs_vec y);                     /* y = 1 / x   */
FS_API int fs_vec_linear_sum(double alpha, fs_vec x, double beta, fs_vec y, fs_vec z);
FS_API int fs_vec_axpy(double alpha, fs_vec x, fs_vec y, fs_vec z);   /* z = alpha x + y, core.hh:189 */
FS_API int fs_vec_axpby(double alpha, double beta, fs_vec x, fs_vec z); /* z = alpha x + beta z */
FS_API int fs_vec_abs(fs_vec x, fs_vec y);                            /* y = |x|     */
FS_API int fs_vec_add_scalar(fs_vec x, double alpha, fs_vec y);       /* y = x + alpha */
/* set_random(seed), core.hh:302-310: uniform [0,1) from splitmix64(seed) */
FS_API int fs_vec_set_random(fs_vec x, uint64_t seed);

/* Reductions (core.hh:229-290).  Deterministic: a fixed-order block tree,
 * the same bits for the same inputs on the same device.  Single-precision
 * vectors accumulate with compensated (two-sum / two-product) arithmetic. */
FS_API int fs_vec_dot(fs_vec x, fs_vec y, double *out);
FS_API int fs_vec_l1norm(fs_vec x, double *out);
FS_API int fs_vec_l2norm(fs_vec x, double *out);
FS_API int fs_vec_inf_norm(fs_vec x, double *out);
FS_API int fs_vec_min(fs_vec x, double *out);
FS_API int fs_vec_max(fs_vec x, double *out);

/* --------------------------------------------------------- matrices --- */
/* Device CSR operator: replaces mat::sparse / compressed_ops::spmv
 * (flecsolve/matrices/seq.hh:35-63, 177-193).  rowptr has nrows+1 offsets,
 * col holds column ids of width index_bytes (4 or 8; the reference's
 * mat::csr<double> uses std::size_t), val holds doubles.  The library stores
 * int32 column ids and keeps a float copy of the values for mixed precision. */
FS_API int fs_csr_create(fs_ctx ctx, int64_t nrows, int64_t ncols, int64_t nnz,
                         const int64_t *rowptr, const void *col, int index_bytes,
                         const double *val, fs_csr *out);
FS_API int fs_csr_destroy(fs_csr A);
FS_API int fs_csr_shape(fs_csr A, int64_t *nrows, int64_t *ncols, int64_t *nnz);
/* overwrite the values (same pattern) from host memory */
FS_API int fs_csr_update_values(fs_csr A, const double *val);
/* overwrite the values from device memory (float64, nnz entries) */
FS_API int fs_csr_update_values_device(fs_csr A, const double *dval);
FS_API int fs_csr_values_device_ptr(fs_csr A, double **dval);
/* Index coding (no counterpart in the reference; a storage choice of this
 * library).  All formats give identical results.
 *  0 column ids: 32-bit column id per nonzero.
 *  1 row patterns: when every row has at most 8 nonzeros and the matrix has at
 *    most 256 distinct sequences of column offsets c - r (stencil operators),
 *    one byte per row names its sequence; neither column ids nor row offsets
 *    are read.
 *  2 symmetric storage: row patterns of a square matrix whose values are
 *    symmetric bit for bit are read from the diagonal and the upper diagonals
 *    only (a(r, r-d) = a(r-d, r)).  Derived from the current values and
 *    checked whenever they change; an asymmetric matrix uses format 1.
 *  3 grid stencil (the default): the symmetric storage of a 1-, 2- or 3-D
 *    grid stencil (positive offsets 1, nx, nx ny; every row holds exactly its
 *    neighbours inside the grid, found at creation) with nx a multiple of 4:
 *    rows are addressed by their grid coordinates, no pattern id is read, and
 *    16-byte loads serve 4 (FP32) or 2 (FP64) rows.  Other matrices use
 *    format 2.
 *  4 general grid stencil (active only, through a request of format 3): a
 *    grid stencil as in format 3 whose values are not symmetric, read from
 *    the diagonal, the upper diagonals and the lower diagonals a(r, r - d)
 *    stored at row r.
 *  Formats 1-4 give the bits of format 0.
 * enable: 0 .. 3 requests a format (a matrix falls back to the best format it
 * supports), -1 leaves it unchanged; *active (may be NULL) = the format the
 * FP64 SpMV uses now. */
FS_API int fs_csr_index_coding(fs_csr A, int enable, int *active);
/* the grid of a grid-stencil matrix (format 3): dims = {nx, ny, nz}, all 0
 * when the matrix is none; no counterpart in the reference */
FS_API int fs_csr_grid_dims(fs_csr A, int64_t dims[3]);
/* number of SpMV row blocks (at most 256 rows and 1792 nonzeros each, a
 * longer row alone); no counterpart in the reference */
FS_API int fs_csr_row_blocks(fs_csr A, int64_t *nblk);
/* Kernel of the FMA-mode column-id SpMV for values of `dtype` (no
 * counterpart in the reference; a schedule choice of this library): 0 the
 * row-block kernel (one thread per row), 4 / 8 / 16 / 32 the vector kernel
 * with that many lanes per row, 1 the vector kernel with the rows binned by
 * length (4 to 32 lanes per row by class).  Matrices with row patterns (stencil
 * operators, formats 1-3) always keep the row formats; EXACT mode always
 * sums each row in one thread, in the reference's order.
 * fs_csr_tune times every candidate on the context's stream (synchronising
 * it) and keeps the fastest; an untuned matrix is tuned by its first SpMV
 * outside a CUDA-graph capture (inside one, the mean row length chooses).
 * *lanes (may be NULL) = the choice.  fs_csr_set_lanes fixes the choice; -1
 * drops it so that the next SpMV tunes again. */
FS_API int fs_csr_tune(fs_csr A, int dtype, int *lanes);
FS_API int fs_csr_set_lanes(fs_csr A, int dtype, int lanes);

/* ---------------------------------------------- MatrixMarket input ----
 * Host only: no context or device needed.  Reads a MatrixMarket coordinate
 * file into CSR exactly as mat::io::matrix_market<double>::read(file)
 * .tocsr() does (flecsolve/matrices/io/matrix_market.hh:31-123,
 * coo::tocsr matrices/seq.hh:324-352):
 *  - a "symmetric" anywhere in the header lines (also "skew-symmetric")
 *    mirrors every off-diagonal entry with the same value, right after it;
 *  - sizes are the atoi of the first three ' '-separated fields of the first
 *    line not starting with '%';
 *  - entries are ' '-separated "row col value" (1-based) read with
 *    std::stoi / std::stof: values are rounded to float, then widened; a
 *    missing value repeats the column field (the reference reads all three
 *    fields into one string);
 *  - rows keep the file order of their entries, duplicates included.
 * A file the reference's reader throws on (an empty or non-numeric field, a
 * value outside the float range, too few entry lines) returns FS_ERR_IO, as
 * does a row or column id outside the matrix. */
FS_API int fs_mm_read(const char *path, fs_mm *out);
/* rows, columns, stored entries (after mirroring), symmetric flag */
FS_API int fs_mm_shape(fs_mm m, int64_t *nrows, int64_t *ncols, int64_t *nnz, int *symmetric);
/* Rows [row_begin, row_end) in CSR, as matrix_market::definition::matrix(range)
 * cuts them (matrix_market.hh:126-156): rowptr (row_end - row_begin + 1
 * entries) relative to the range's first entry, global column ids, values.
 * Any array may be NULL; *nnz_out (may be NULL) = entries in the range.
 * [0, nrows) is the whole matrix, ready for fs_csr_create (index_bytes 8). */
FS_API int fs_mm_rows(fs_mm m, int64_t row_begin, int64_t row_end, int64_t *rowptr,
                      int64_t *col, double *val, int64_t *nnz_out);
FS_API int fs_mm_destroy(fs_mm m);

/* SpMV modes */
enum fs_spmv_mode {
	FS_SPMV_FMA = 0,      /* y_i accumulated with fused multiply-add      */
	FS_SPMV_EXACT = 1     /* products rounded, then summed left to right:
	                         the reference's row loop bit for bit         */
};
/* y = A x (op::core::apply -> mat::sparse::apply, matrices/seq.hh:50-60).
 * x and y are both FS_F64 or both FS_F32 (FS_F32 uses the float values). */
FS_API int fs_csr_spmv(fs_csr A, fs_vec x, fs_vec y, int mode);
/* r = b - A x (op::core::residual, operators/core.hh:129-142) */
FS_API int fs_csr_residual(fs_csr A, fs_vec b, fs_vec x, fs_vec r);
/* y = A^T x through a precomputed CSC view (atomic-free); the view is built
 * on first use and kept until the values or the matrix change */
FS_API int fs_csr_spmv_transpose(fs_csr A, fs_vec x, fs_vec y);
/* dinv_i = 1 / a_ii, the D^-1 operator of flecsolve/util/test/mesh.hh:123-140 */
FS_API int fs_csr_diag_inv(fs_csr A, fs_vec dinv);

/* Caller-defined operator: op::make_shell / op::base
 * (flecsolve/operators/shell.hh:26-95, operators/core.hh:29-78).  The
 * callback computes y = Op(x) for FS_F64 device vectors of the operator's
 * context, on the host thread that called the library, and returns 0 on
 * success (anything else stops the caller's solve with FS_ERR_CALLBACK).  It
 * may call any fs_* function on the context (SpMVs, vector ops, a bound
 * solver's apply) or launch its own kernels.  The library drains the
 * context's stream before each call, so x is complete; the callback returns
 * once y is written, or once the work that writes y is enqueued on the
 * context's stream (fs_ctx_stream; every fs_* call on the context is).  The
 * handle is an fs_csr that stores no rows: fs_csr_spmv / fs_csr_residual and
 * every Krylov solver (as A or as the preconditioner) take it; the calls that
 * need stored values (value updates, transposes, index formats, parcsr,
 * batched and block solves, Jacobi of it) return FS_ERR_INVALID_ARG.  Destroy
 * with fs_csr_destroy. */
typedef int (*fs_op_fn)(void *user, fs_vec x, fs_vec y);
FS_API int fs_shell_create(fs_ctx ctx, int64_t nrows, int64_t ncols, fs_op_fn fn, void *user,
                           fs_csr *out);

/* Row-block distributed SpMV of mat::parcsr (flecsolve/matrices/parcsr.hh:
 * 60-91, topo/csr.hh:482-618): rows are split into `parts` contiguous blocks
 * as flecsi::util::equal_map splits them (parcsr.hh:149-151: blocks of
 * nrows / parts rows, the first nrows % parts one row longer), each row's
 * owned-column (diag block) and ghost-column (offd block) entries are summed
 * separately and added, y = y_diag + y_offd.  All parts live on this
 * device. */
FS_API int fs_parcsr_spmv(fs_csr A, int parts, fs_vec x, fs_vec y);

/* One color of the distributed operator itself: mat::parcsr over topo::csr
 * (flecsolve/matrices/parcsr.hh:29-177, topo/csr.hh:413-632), the color's
 * rows on this device.  From the color's rows (rowptr[nrows + 1], global
 * column ids gcol, values) and its owned column block [col_begin, col_end)
 * (the column block of the same color, an equal_map block as in
 * parcsr.hh:166-169), built as the reference's coloring and init_mats build
 * it (csr.hh:482-618): the ghost columns are the column ids outside the
 * owned block, sorted and unique (the colmap, fs_parcsr_ghosts); the diag
 * part holds the owned entries (column = id - col_begin), the offd part the
 * ghost entries (column = nown + the ghost's position in the colmap), each
 * row in input order.
 * fs_parcsr_color_spmv: y = diag x + offd x (parcsr.hh:60-71) for x holding
 * the color's columns -- its nown owned values, then one value per ghost in
 * colmap order, filled by the caller's halo exchange from the owning colors
 * (topo/csr.hh:240-304).  Each row's diag and offd sums are taken
 * separately with the reference's row arithmetic and then added: the bits
 * of fs_parcsr_spmv on the whole matrix. */
FS_API int fs_parcsr_create(fs_ctx ctx, int64_t col_begin, int64_t col_end, int64_t nrows,
                            const int64_t *rowptr, const int64_t *gcol, const double *val,
                            fs_parcsr *out);
FS_API int fs_parcsr_destroy(fs_parcsr A);
FS_API int fs_parcsr_shape(fs_parcsr A, int64_t *nrows, int64_t *nown, int64_t *nghost,
                           int64_t *nnz_diag, int64_t *nnz_offd);
/* the colmap: *n in = capacity (gids may be NULL to query), out = count */
FS_API int fs_parcsr_ghosts(fs_parcsr A, int64_t *gids, int64_t *n);
FS_API int fs_parcsr_color_spmv(fs_parcsr A, fs_vec x, fs_vec y);

/* ---------------------------------------------------------- solvers --- */
/* solver_settings, flecsolve/solvers/solver_settings.hh:31-36 */
typedef struct {
	int maxiter;
	float rtol;
	float atol;          /* accepted and unused, as in the reference */
	int use_zero_guess;
} fs_solver_settings;

/* solve_info, flecsolve/solvers/solver_settings.hh:61-85 */
typedef struct {
	int status;          /* enum fs_stop_reason */
	int iters;
	int restarts;
	float res_norm_initial, res_norm_final;
	float sol_norm_initial, sol_norm_final;
	float rhs_norm;
} fs_solve_info;

enum fs_method {
	FS_CG = 0,           /* op::cg, cg.hh:43-139                         */
	FS_BICGSTAB = 1,     /* op::bicgstab, bicgstab.hh:39-187             */
	FS_GMRES = 2,        /* op::gmres, gmres.hh:78-241                   */
	FS_CG_MIXED = 3,     /* FP32 inner PCG inside FP64 refinement        */
	FS_BICGSTAB_MIXED = 4, /* FP32 BiCGSTAB, FP64 residual replacement   */
	FS_GMRES_MIXED = 5,  /* FP32 Arnoldi cycles, FP64 restart residual   */
	FS_FCG = 6,          /* op::fcg, flexible CG, cg.hh:145-244          */
	FS_CG_PIPELINED = 7  /* op::cg's recurrences rearranged (Chronopoulos
	                        & Gear) to one grid reduction per iteration    */
};

/* The preconditioner slot P of krylov_parameters (krylov_parameters.hh:
 * 41-78): any operator.  Identity, Jacobi and diagonal preconditioners (and
 * a CSR whose entries are all on the diagonal, the reference's D^-1
 * operator) are fused into the device loops of every method; any other
 * operator -- a general CSR, a matrix-free or shell handle, a bound solver
 * (the NKA / nested-solver pattern of solvers/test/nka.cc:72-80) -- is
 * applied as its own step of host-stepped loops that follow the reference's
 * operation order (FP64 methods and FS_FCG; the mixed methods return
 * FS_ERR_UNSUPPORTED for it). */
enum fs_precond_kind {
	FS_PRECOND_NONE = 0,   /* op::I, operators/shell.hh:94-95             */
	FS_PRECOND_JACOBI = 1, /* D^-1 of A (util/test/mesh.hh:123-140)       */
	FS_PRECOND_DIAG = 2,   /* caller-given diagonal vector (z_i = d_i r_i) */
	FS_PRECOND_CSR = 3,    /* an fs_csr operator: z = P r                  */
	FS_PRECOND_SOLVER = 4  /* a bound solver: z = solve(r) with its own
	                          settings, operator and preconditioner         */
};

typedef struct {
	int kind;            /* enum fs_precond_kind */
	fs_vec diag;         /* FS_PRECOND_DIAG      */
	fs_csr op;           /* FS_PRECOND_CSR       */
	fs_solver solver;    /* FS_PRECOND_SOLVER    */
} fs_precond;

enum fs_gmres_side { FS_LEFT = 0, FS_RIGHT = 1 };
/* GMRES orthogonalisation.  AUTO picks MGS for the FP64 basis (half the FP64
 * multiply-adds of CGS2, and the reference's order) and DCGS2 (below; CGS2
 * where DCGS2 cannot run) for the FP32 basis of FS_GMRES_MIXED: 2 passes and
 * 1 reduction per step instead of the k + 2 of MGS.
 * DCGS2: CGS2 with each vector's reorthogonalisation delayed to the next
 * step, where it shares that step's pass of dot products (two passes over
 * the basis a step instead of three); the convergence test of a step runs
 * one SpMV later.  It needs the staged passes (m <= 30 and a basis the tensor
 * unit can address) and, for FS_GMRES, no diagnostic callback; otherwise
 * CGS2 runs. */
enum fs_gmres_ortho { FS_ORTHO_CGS2 = 0, FS_ORTHO_MGS = 1, FS_ORTHO_AUTO = 2, FS_ORTHO_DCGS2 = 3 };

enum fs_refine_kind {
	FS_REFINE_RESTART = 0,  /* outer FP64 residual, inner FP32 PCG restarted */
	FS_REFINE_RELIABLE = 1  /* FP32 recurrences with FP64 residual
	                           replacement, search direction kept          */
};

/* Krylov settings: the reference's per-solver settings in one struct
 * (cg.hh:254, bicgstab.hh:197, gmres.hh:389-405) plus the device controls. */
typedef struct {
	fs_solver_settings base;
	/* GMRES (gmres.hh:389-422) */
	int max_krylov_dim;  /* -1 = maxiter; bound 100 */
	int pre_side;        /* enum fs_gmres_side */
	int restart;
	int ortho;           /* enum fs_gmres_ortho */
	/* device loop: iterations per CUDA-graph launch between residual
	   read-backs (0 = library default) */
	int k_readback;
	/* mixed precision (FS_*_MIXED); default FS_REFINE_RELIABLE */
	int refine;          /* enum fs_refine_kind */
	double inner_rtol;   /* restart: inner relative tolerance (0 = 1e-4);
	                        reliable: residual reduction between FP64
	                        replacements (0 = 0.1 for CG and batched CG,
	                        1e-2 for BiCGSTAB)                              */
	int max_outer;       /* restart: maximum refinement steps            */
	/* reliable mixed CG and batched CG: FP64 iterations until the residual
	   is below fp64_head * ||b||, then FP32 recurrences with FP64
	   replacement for the rest of the same Krylov process (default 3e-3;
	   0 = FP32 from the first iteration).  The solution's large components
	   form in the first decades of residual reduction.  Computed in FP32,
	   they cost the iterates orthogonality (up to 118 more iterations than
	   FP64 on 2-D log-normal diffusion systems of 256^2; 90 with a head of
	   1e-2) and put the result 1.8e-8 from the FP64 solve's iterate at
	   256^3 (1e-2: 1.2e-8).  The default head gives 4e-9 there and the FP64
	   iteration count within 2 on all 512 batched systems. */
	double fp64_head;
} fs_krylov_settings;

/* Fill `s` with the reference defaults (gmres.hh:414-418) and device defaults. */
FS_API int fs_krylov_settings_default(fs_krylov_settings *s);

/* The diagnostic callable bool(const Vec &, double) of the reference
 * (cg.hh:112, bicgstab.hh:160, gmres.hh:196).  Nonzero return stops the
 * solve with FS_CONVERGED_USER. */
typedef int (*fs_diag_fn)(void *user, fs_vec x, double res_norm);

/* Bind a solver: krylov_solver::bind / operator() (krylov_parameters.hh:94-
 * 126) -- settings, work vectors (make_work, solver_settings.hh:189-200), the
 * operator and the preconditioner.  The solver owns its work vectors and
 * its captured CUDA graphs. */
FS_API int fs_krylov_create(fs_ctx ctx, int method, const fs_krylov_settings *s,
                            fs_csr A, const fs_precond *P, fs_solver *out);
FS_API int fs_krylov_destroy(fs_solver s);
FS_API int fs_krylov_set_diagnostic(fs_solver s, fs_diag_fn fn, void *user);
FS_API int fs_krylov_settings_get(fs_solver s, fs_krylov_settings *out);
FS_API int fs_krylov_settings_set(fs_solver s, const fs_krylov_settings *in);
/* op::core::apply(b, x) of the bound solver (operators/core.hh:107-116) */
FS_API int fs_krylov_apply(fs_solver s, fs_vec b, fs_vec x, fs_solve_info *info);
/* per-iteration residual norms of the last apply (the values handed to the
 * diagnostic); n on input = capacity, on output = count written */
FS_API int fs_krylov_history(fs_solver s, double *hist, int64_t *n);
/* number of refinement (outer) steps and total inner iterations of the last
 * FS_CG_MIXED apply */
FS_API int fs_krylov_mixed_stats(fs_solver s, int *outer, int *inner_iters);

/* ------------------------------------------------------------ adjoint --- */
/* No counterpart in the reference (it has no adjoint).  For a loss L(x) of
 * x = A^-1 b:  A^T lambda = dL/dx (fs_krylov_apply_transpose: the bound
 * solver on the transposed operator, a CSC view of A built once per pattern),
 * dL/db = lambda, dL/dA_ij = -lambda_i x_j (fs_csr_value_grad), and for the
 * finite-volume diffusion operator assembled from face coefficients
 * (fs_fv_assemble, same face layout and row order as the seeded generators)
 * dL/dc_f = -(lambda_i - lambda_j)(x_i - x_j), or -lambda_i x_i on the
 * boundary (fs_fv_face_grad; `scale` multiplies, `accumulate` adds to g). */
FS_API int fs_krylov_apply_transpose(fs_solver s, fs_vec b, fs_vec x, fs_solve_info *info);
FS_API int fs_csr_transpose(fs_csr A, fs_csr *AT);
FS_API int fs_csr_value_grad(fs_csr A, fs_vec lambda, fs_vec x, fs_vec grad_values);
/* A.values = scale * K(faces) + shift * I for an n^dim grid (dim 2 or 3) */
FS_API int fs_fv_assemble(fs_csr A, int dim, int64_t n, fs_vec faces, double scale, double shift);
FS_API int fs_fv_face_grad(fs_ctx ctx, int dim, int64_t n, fs_vec lambda, fs_vec x, double scale,
                           int accumulate, fs_vec grad_faces);

/* --------------------------------------------------- batched solves --- */
/* Many independent systems in one persistent launch (no counterpart in the
 * reference, whose solvers take one system per call: this batches calls of
 * cg.hh:43-139).  A is block diagonal: system s owns rows and columns
 * [sys_offsets[s], sys_offsets[s+1]).  One thread-block cluster per system
 * runs Jacobi-PCG with FP32 values/vectors and FP64 residual replacement
 * (settings->inner_rtol = replacement factor), stopping per system on the
 * FP64 residual (rtol * ||b_s||).  cluster_size (1, 2, 4, 8) and threads per
 * CTA may be 0: an autotuner times the candidates on the first call for this
 * partition and keeps the fastest (fs_batch_tuning reports it).  With both 0
 * it also tries schedules where only the largest systems own a whole cluster
 * and every other system one CTA (fs_batch_schedule reports how many own a
 * cluster).  infos[s] receives system s's solve_info. */
FS_API int fs_batch_cg_solve(fs_ctx ctx, const fs_krylov_settings *s, fs_csr A, int nsys,
                             const int64_t *sys_offsets, fs_vec b, fs_vec x, int cluster_size,
                             int threads, fs_solve_info *infos);
FS_API int fs_batch_tuning(fs_ctx ctx, fs_csr A, int nsys, const int64_t *sys_offsets,
                           int *cluster_size, int *threads);
FS_API int fs_batch_schedule(fs_ctx ctx, fs_csr A, int nsys, const int64_t *sys_offsets,
                             int *cluster_size, int *threads, int *cluster_systems);
/* The storage the batched kernel's row sums read for this partition, checked
 * on the first solve after the values change: FS_BATCH_GRID when every
 * system is a 5-point operator on a square s x s grid (rows hold exactly
 * their in-grid neighbours, columns sorted) whose lower entries equal their
 * partners bit for bit -- the diagonal and two upper diagonals are read,
 * no column ids, with the CSR row loop's bits -- else FS_BATCH_CSR. */
#define FS_BATCH_CSR 0
#define FS_BATCH_GRID 1
FS_API int fs_batch_format(fs_ctx ctx, fs_csr A, int nsys, const int64_t *sys_offsets, int *format);
/* the same solve with an explicit schedule: the cluster_systems largest
 * systems own a cluster of cluster_size CTAs, every other system one CTA
 * (cluster_size of them per cluster); sizes must be given */
FS_API int fs_batch_cg_solve_split(fs_ctx ctx, const fs_krylov_settings *s, fs_csr A, int nsys,
                                   const int64_t *sys_offsets, fs_vec b, fs_vec x, int cluster_size,
                                   int threads, int cluster_systems, fs_solve_info *infos);

/* Block Jacobi-PCG for nrhs = 16 right-hand sides of one operator (FP64).
 * No counterpart in the reference (its CG, cg.hh:43-139, takes one
 * right-hand side per call).  B and X hold N x 16 values row-major (the 16
 * values of row r contiguous).  P: NULL/FS_PRECOND_NONE or
 * FS_PRECOND_JACOBI.  Column j converges when ||R_j|| < rtol ||B_j||;
 * infos[j].iters is the block iteration at which it did, infos[j].restarts
 * the block iterations run. */
FS_API int fs_block_cg_solve(fs_ctx ctx, const fs_krylov_settings *s, fs_csr A,
                             const fs_precond *P, int nrhs, fs_vec B, fs_vec X,
                             fs_solve_info *infos);
/* The same with FP32 block recurrences (FP32 matrix values and vectors,
 * compensated FP32 Gram sums) and FP64 residual replacement: the FP64 X is
 * updated and R replaced by B - A X in FP64 whenever every unconverged
 * column's residual has dropped by s->inner_rtol (0 = 0.1) since the last
 * replacement, or a column may have converged; columns converge on the FP64
 * residual only.  B and X are FP64 as above. */
FS_API int fs_block_cg_solve_mixed(fs_ctx ctx, const fs_krylov_settings *s, fs_csr A,
                                   const fs_precond *P, int nrhs, fs_vec B, fs_vec X,
                                   fs_solve_info *infos);

/* ------------------------------------------ allocation-free reduction --- */
/* No counterpart in the reference.  Dot product sum_i x[i] * y[i] of two
 * float64 device arrays, written to the device pointer `result`, for callers
 * that cannot allocate device memory: code whose device memory is owned by
 * another allocator (a framework's caching allocator or a fixed budget),
 * code that cannot take the implicit device synchronisation of cudaMalloc /
 * cudaFree, and code that holds only raw device pointers and a stream (no
 * fs_ctx, whose creation allocates).  It calls no cudaMalloc, cudaFree or
 * allocating library routine: its scratch is a 128 KiB static device array
 * that every GPU loading libfsgpu.so holds until the process exits.
 *  - n <= FS_DOT_NOALLOC_MAX_N (64 Mi elements, one scratch slot per 4096
 *    elements); larger n returns FS_ERR_INVALID_ARG and launches nothing.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream) of the current
 *    device.  The scratch array's device address belongs to a CUDA context:
 *    the first call under each context (the device's primary context, or a
 *    context the caller made current with the driver API) looks it up
 *    (cudaGetSymbolAddress) and caches it for that context; make that first
 *    call before any stream capture.
 *  - Every call shares the one scratch array, so calls whose kernels can
 *    overlap on the GPU (different streams without ordering) race.
 *  - The result is deterministic for a given n and agrees with fs_vec_dot to
 *    rounding (the two group the partial sums differently). */
#define FS_DOT_NOALLOC_MAX_N ((int64_t)67108864)
FS_API int fs_dot_f64_noalloc(const double *x, const double *y, int64_t n,
                              double *result, void *stream);

/* ------------------------------------------------------------- NKA ----
 * Nonlinear Krylov accelerator (Carlson and Miller), op::nka of
 * flecsolve/solvers/nka.hh:31-605, over device vectors.  Settings are
 * nka::settings (nka.hh:518-545): the common solver settings (maxiter,
 * rtol, atol, use_zero_guess) plus the acceleration controls. */
typedef struct {
	fs_solver_settings base;
	int max_dim;            /* acceleration subspace dimension (> 0)            */
	double angle_tol;       /* drop a vector whose factor diagonal <= angle_tol */
	int max_fun_evals;      /* accepted, unused (as in the reference)           */
	int freeze_pc;          /* accepted: a linear F's preconditioner is fixed   */
	int use_qr;             /* not implemented (as in the reference)            */
	int use_damping;
	int adaptive_damping;   /* eta = 1 - 0.9^min(k, max_dim); needs use_damping */
	double damping_factor;
} fs_nka_settings;
/* the reference's option defaults (nka.hh:536-552, solver_settings.hh:40-52);
 * max_dim has none there and is set to 0 (must be set) */
FS_API int fs_nka_settings_default(fs_nka_settings *s);
/* r = f - F(u): the residual of a (nonlinear) operator, op::core::residual */
typedef int (*fs_residual_fn)(void *user, fs_vec f, fs_vec u, fs_vec r);
/* Bind NKA (nka::solver(settings, work)(F, P), nka.hh:587-597): F is a CSR
 * operator, or NULL with `fres` for a nonlinear residual; P is a bound
 * Krylov solver applied as the preconditioner (P.apply(res, correction):
 * solvers/test/nka.cc:72-80 uses CG), or NULL for none.  The solver owns
 * (max_dim + 1) * 2 + 3 work vectors.  Invalid settings return
 * FS_ERR_BREAKDOWN (the reference asserts), use_qr FS_ERR_UNSUPPORTED. */
FS_API int fs_nka_create(fs_ctx ctx, const fs_nka_settings *s, fs_csr F, fs_residual_fn fres,
                         void *fres_user, fs_solver P, fs_nka *out);
FS_API int fs_nka_set_diagnostic(fs_nka k, fs_diag_fn fn, void *user);
/* op::nka::apply(f, u) (nka.hh:64-137).  The acceleration subspace persists
 * across applies, as the reference's does; fs_nka_reset empties it.  A solve
 * that runs out of iterations leaves status FS_STATUS_UNKNOWN and iters 0. */
FS_API int fs_nka_apply(fs_nka k, fs_vec f, fs_vec u, fs_solve_info *info);
FS_API int fs_nka_reset(fs_nka k);
FS_API int fs_nka_destroy(fs_nka k);

/* ------------------------------------------- finite-volume physics ----
 * The structured-mesh physics operators of flecsolve/physics/: boundary
 * operators, face-coefficient setters and the volume diffusion operator
 *   v = -beta div(b grad u) + alpha vol a u
 * (volume_diffusion/diffusion.hh:59-262), on the device.
 *
 * Mesh: n[0] x n[1] x n[2] (x, y, z) logical cells on the box [box[a][0],
 * box[a][1]] per axis, with one layer of boundary cells on every side, as
 * the reference's fvm_narray with boundary depth 1 (physics/test/
 * test_setup.hh:47-74).  Spacing, face areas and cell volume follow the
 * specialization (physics/specializations/fvm_narray.hh:233-289):
 * dx = |hi - lo| / (n + 1).
 *  - a cell field is (n[2]+2)(n[1]+2)(n[0]+2) doubles, [k][j][i] with i
 *    fastest, logical cells 1..n per axis;
 *  - a face field (one per axis) is (n[2]+1)(n[1]+1)(n[0]+1) doubles in the
 *    same order; face i of an axis lies between cells i and i+1 of it;
 *  - a vector of logical cells (the solvers' vectors) is n[0] n[1] n[2]
 *    doubles or floats, i fastest (the reference vectors' degrees of
 *    freedom).
 * Every field is an FP64 fs_vec of the context's device. */
enum {
	FS_FVM_X_LOW = 0, FS_FVM_X_HIGH = 1, FS_FVM_Y_LOW = 2,
	FS_FVM_Y_HIGH = 3, FS_FVM_Z_LOW = 4, FS_FVM_Z_HIGH = 5
};
enum { FS_BC_NONE = 0, FS_BC_DIRICHLET = 1, FS_BC_NEUMANN = 2 };
typedef struct {
	int64_t n[3];
	double box[3][2];
} fs_fvm_mesh;
/* dx, face areas dA (normal_dA) and the cell volume of the mesh (any may be
 * NULL) */
FS_API int fs_fvm_geometry(const fs_fvm_mesh *m, double dx[3], double dA[3], double *volume);
/* bc<dirichlet, axis, boundary> / bc<neumann, ...>::apply on the cell field
 * u (boundary/dirichlet.hh:49-63: the boundary cells get `value`;
 * boundary/neumann.hh:49-74: they get the neighbouring cell minus
 * (nd dx) value, nd = +1 on a low face, -1 on a high one) */
FS_API int fs_fvm_boundary(fs_ctx ctx, const fs_fvm_mesh *m, int face, int kind, double value, fs_vec u);
/* coefficient<constant_coefficient> / coefficient<average_coefficient>::
 * apply (volume_diffusion/coefficient.hh:84-177): the face fields get
 * `value`, or the average 0.5 (u_hi + u_lo) of the cells either side */
FS_API int fs_fvm_coef_constant(fs_ctx ctx, const fs_fvm_mesh *m, double value, fs_vec bx, fs_vec by,
                                fs_vec bz);
FS_API int fs_fvm_coef_average(fs_ctx ctx, const fs_fvm_mesh *m, fs_vec u, fs_vec bx, fs_vec by, fs_vec bz);
/* diffusion::apply (diffusion.hh:83-107, 109-193): v on the logical cells
 * from the cell fields a, u and the face fields b (its boundary cells are
 * left as they are); the same values as the reference bit for bit */
FS_API int fs_fvm_diffusion(fs_ctx ctx, const fs_fvm_mesh *m, double beta, double alpha, fs_vec a, fs_vec bx,
                            fs_vec by, fs_vec bz, fs_vec u, fs_vec v);
/* the logical cells of a cell field as a vector, and back */
FS_API int fs_fvm_pack(fs_ctx ctx, const fs_fvm_mesh *m, fs_vec field, fs_vec x);
FS_API int fs_fvm_unpack(fs_ctx ctx, const fs_fvm_mesh *m, fs_vec x, fs_vec field);

/* Matrix-free operator: the expression op_expr(six boundary operators,
 * a face coefficient, diffusion) as an operator on vectors of logical cells,
 * returned as an fs_csr handle that stores no rows.  fs_csr_spmv,
 * fs_csr_residual, fs_csr_diag_inv, fs_csr_shape, fs_csr_destroy and every
 * Krylov solver (FP64, FP32 and mixed) accept it; the calls that need stored
 * values (updates, transposes, index formats, parcsr, block and batched
 * solves) return FS_ERR_INVALID_ARG.  Per cell the apply gives the values
 * fs_fvm_diffusion gives on a field whose boundary cells the six boundary
 * operators set.  A Dirichlet value or Neumann flux other than 0 makes the
 * operator affine (A(0) != 0), as the reference's is. */
typedef struct {
	fs_fvm_mesh mesh;
	double beta, alpha;
	int bc_kind[6];      /* per face (FS_FVM_*): FS_BC_DIRICHLET or FS_BC_NEUMANN */
	double bc_value[6];  /* boundary_value / flux_value                          */
	double a_value;      /* the cell coefficient a when the field a is NULL      */
	double b_value;      /* the face coefficient when the face fields are NULL   */
} fs_fvm_operator_settings;
/* The face and cell coefficients are copied (as transmissibilities t = b dA /
 * dx and (alpha vol) a) when the operator is created; the fields may be
 * destroyed afterwards, and changing them needs a new operator. */
FS_API int fs_fvm_operator_create(fs_ctx ctx, const fs_fvm_operator_settings *s, fs_vec a, fs_vec bx,
                                  fs_vec by, fs_vec bz, fs_csr *out);
/* whether the operator is affine, and its logical cells per axis */
FS_API int fs_fvm_operator_info(fs_csr A, int *affine, int64_t n[3]);

/* ------------------------------------------------- BDF integrator ----
 * bdf::integrator of flecsolve/time-integrators/bdf.hh:49-777 for
 * u' = f(u): backward Euler, Crank-Nicolson and variable-step BDF2-6 with
 * AB2 / leapfrog / forward-Euler predictors, truncation-error estimates and
 * the PI / deadbeat step controllers.  The controller runs on the host; every
 * vector operation (predictor, source term, error estimate, history) and the
 * solve of the time operator u - gamma f(u) = rhs run on the device.
 * Settings are bdf::settings (bdf_parameters.hh:35-112) with the enums of
 * bdf_parameters.hh:16-24 in their declaration order. */
typedef struct fs_bdf_s *fs_bdf;
enum { FS_BDF_CN = 0, FS_BDF_BE = 1, FS_BDF_BDF2 = 2, FS_BDF_BDF3 = 3, FS_BDF_BDF4 = 4,
       FS_BDF_BDF5 = 5, FS_BDF_BDF6 = 6 };
enum { FS_BDF_AB2 = 0, FS_BDF_LEAPFROG = 1 };
enum { FS_BDF_TRUNCATION_ERROR = 0, FS_BDF_CONSTANT = 1, FS_BDF_FINAL_CONSTANT = 2,
       FS_BDF_LIMIT_RELATIVE_CHANGE = 3 };
enum { FS_BDF_H211B = 0, FS_BDF_PC4_7 = 1, FS_BDF_PC11 = 2, FS_BDF_DEADBEAT = 3 };
enum { FS_BDF_FIXED_RESOLUTION = 0, FS_BDF_FIXED_SCALING = 1 };
enum { FS_NORM_INF = 0, FS_NORM_L2 = 1, FS_NORM_L1 = 2 };  /* vec::norm_type */
typedef struct {
	/* time_integrator::base_settings (parameters.hh:21-28) */
	double initial_time, final_time;
	int max_steps;
	double max_dt, min_dt, initial_dt;
	/* bdf::settings */
	int use_predictor, use_initial_predictor, has_source_term, combine_timestep_estimators;
	int predictor;                 /* FS_BDF_AB2 / FS_BDF_LEAPFROG */
	int timestep_strategy;         /* FS_BDF_TRUNCATION_ERROR ... */
	double dt_cut_lower_bound, dt_growth_upper_bound;
	int number_of_time_intervals;
	int integrator, starting_integrator;  /* FS_BDF_CN ... FS_BDF_BDF6 */
	int calculate_time_trunc_error;
	int time_trunc_err_norm;       /* FS_NORM_* (inf, else the l2 norm) */
	double target_relative_change;
	int use_pi_controller, pi_controller_type, control_timestep_variation;
	int time_error_scaling;        /* FS_BDF_FIXED_RESOLUTION / _SCALING */
	double time_rtol, time_atol;
	int num_problem_scales;        /* 0 or 1: problem_scales of one component */
	double problem_scale;
} fs_bdf_settings;
/* the option defaults of bdf::options (bdf_parameters.hh:121-156); the
 * options without a default there (times, max_steps, predictor, strategy,
 * integrators) are set to -1 and must be given */
FS_API int fs_bdf_settings_default(fs_bdf_settings *s);
/* the time operator of a general problem: f = f(u) (apply_rhs,
 * operator_adapter.hh:40-43), and the solve of x - gamma f(x) = rhs from the
 * initial guess in x (the integrator's solver); *success as
 * solve_info::success() */
typedef int (*fs_rhs_fn)(void *user, fs_vec u, fs_vec f);
typedef int (*fs_time_solve_fn)(void *user, double gamma, fs_vec rhs, fs_vec x, int *success);
/* bdf::integrator(bdf::parameters(settings, op, make_work(x), solver)) for
 * vectors of n doubles.  Invalid settings return FS_ERR_BREAKDOWN (the
 * reference asserts in settings::validate, bdf_parameters.hh:57-110). */
FS_API int fs_bdf_create(fs_ctx ctx, const fs_bdf_settings *s, int64_t n, fs_rhs_fn rhs, void *rhs_user,
                         fs_time_solve_fn solve, void *solve_user, fs_bdf *out);
/* A linear problem f(u) = J u: the time operator I - gamma J is kept as a
 * CSR with J's pattern (J must store its diagonal), its values rewritten on
 * the device whenever gamma changes, and solved by a Krylov solver bound to
 * it (method, settings and preconditioner as fs_krylov_create).  J is read at
 * every step and must outlive the integrator. */
FS_API int fs_bdf_create_linear(fs_ctx ctx, const fs_bdf_settings *s, fs_csr J, int method,
                                const fs_krylov_settings *ks, const fs_precond *P, fs_bdf *out);
/* integrator::advance / check_solution / update / get_next_dt
 * (bdf.hh:74-213): out = the solution at t + dt from curr (curr != out) */
FS_API int fs_bdf_advance(fs_bdf b, double dt, int first_step, fs_vec curr, fs_vec out);
FS_API int fs_bdf_check_solution(fs_bdf b, int *passed);
FS_API int fs_bdf_update(fs_bdf b);
FS_API int fs_bdf_get_next_dt(fs_bdf b, int good_solution, double *dt);
typedef struct {
	double current_time, current_dt, final_time;
	int current_step, num_step_rejects;
	int solver_success;     /* of the last advance */
	int solver_iters;       /* of the last advance (linear form) */
	double gamma;           /* the time operator's scaling of the last step */
} fs_bdf_state;
FS_API int fs_bdf_state_get(fs_bdf b, fs_bdf_state *out);
FS_API int fs_bdf_destroy(fs_bdf b);

#ifdef __cplusplus
}
#endif
#endif
