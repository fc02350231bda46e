// Adjoint of the linear solve x = A(theta)^-1 b.
//
// For a loss L(x): the adjoint solve A^T lambda = dL/dx reuses the bound
// device solver on the transposed operator (a CSC view of A materialised as a
// CSR matrix, built once per pattern and refreshed from the values on use;
// the transpose SpMV is atomic-free), and then
//   dL/db       = lambda
//   dL/dA_ij    = -lambda_i x_j            on the sparsity pattern
//   dL/dc_f     = -(lambda_i - lambda_j)(x_i - x_j)   interior face f = (i, j)
//                 -lambda_i x_i                       boundary face of cell i
// for the finite-volume diffusion operator A(c) = sum_f c_f (e_i - e_j)
// (e_i - e_j)^T (+ c_f e_i e_i^T on the boundary), whose values this file
// also assembles on the device from the face coefficients (the face layout
// and the row order of csrc/problems.c).
#include <cmath>
#include <cstring>

#include "solver.cuh"

namespace fsg {

int ensure_transpose(Csr *A);

namespace {

#define FOR_EACH(i, n)                                                          \
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n);  \
	     i += (int64_t)gridDim.x * blockDim.x)

// face index helpers (same layout as csrc/problems.c)
__device__ __forceinline__ int64_t fx3(int64_t n, int64_t i, int64_t j, int64_t k) {
	return (k * n + j) * (n + 1) + i;
}
__device__ __forceinline__ int64_t fy3(int64_t n, int64_t i, int64_t j, int64_t k) {
	return n * n * (n + 1) + (k * (n + 1) + j) * n + i;
}
__device__ __forceinline__ int64_t fz3(int64_t n, int64_t i, int64_t j, int64_t k) {
	return 2 * n * n * (n + 1) + (k * n + j) * n + i;
}
__device__ __forceinline__ int64_t fx2(int64_t n, int64_t i, int64_t j) { return j * (n + 1) + i; }
__device__ __forceinline__ int64_t fy2(int64_t n, int64_t i, int64_t j) { return n * (n + 1) + j * n + i; }

// A.values = scale * K(c) + shift * I, row order and in-row order of the
// generator (-z, -y, -x, diag, +x, +y, +z); one thread per row
__global__ void k_fv_assemble(int dim, int64_t n, const double *__restrict__ c,
                              const int *__restrict__ rp, double *__restrict__ val, double scale,
                              double shift) {
	const int64_t N = dim == 2 ? n * n : n * n * n;
	FOR_EACH(r, N) {
		int64_t off = rp[r];
		if (dim == 2) {
			const int64_t i = r % n, j = r / n;
			const double cs = c[fy2(n, i, j)], cn = c[fy2(n, i, j + 1)];
			const double cw = c[fx2(n, i, j)], ce = c[fx2(n, i + 1, j)];
			double d = 0.0;
			d += cs;
			d += cw;
			d += ce;
			d += cn;
			if (j > 0) val[off++] = -scale * cs;
			if (i > 0) val[off++] = -scale * cw;
			val[off++] = scale * d + shift;
			if (i + 1 < n) val[off++] = -scale * ce;
			if (j + 1 < n) val[off++] = -scale * cn;
		}
		else {
			const int64_t i = r % n, j = (r / n) % n, k = r / (n * n);
			const double cb = c[fz3(n, i, j, k)], ct = c[fz3(n, i, j, k + 1)];
			const double cs = c[fy3(n, i, j, k)], cn = c[fy3(n, i, j + 1, k)];
			const double cw = c[fx3(n, i, j, k)], ce = c[fx3(n, i + 1, j, k)];
			double d = 0.0;
			d += cb;
			d += cs;
			d += cw;
			d += ce;
			d += cn;
			d += ct;
			if (k > 0) val[off++] = -scale * cb;
			if (j > 0) val[off++] = -scale * cs;
			if (i > 0) val[off++] = -scale * cw;
			val[off++] = scale * d + shift;
			if (i + 1 < n) val[off++] = -scale * ce;
			if (j + 1 < n) val[off++] = -scale * cn;
			if (k + 1 < n) val[off++] = -scale * ct;
		}
	}
}

// gradient of L w.r.t. the face coefficients, one thread per face:
// g_f = -scale * (lam_a - lam_b)(x_a - x_b) for the interior face between
// cells a (lower) and b (upper), -scale * lam_a x_a for a boundary face
__global__ void k_fv_face_grad(int dim, int64_t n, const double *__restrict__ lam,
                               const double *__restrict__ x, double *__restrict__ g, double scale,
                               int accumulate) {
	const int64_t nf = dim == 2 ? 2 * n * (n + 1) : 3 * n * n * (n + 1);
	FOR_EACH(f, nf) {
		int64_t a = -1, b = -1;  // cells on the lower / upper side
		if (dim == 2) {
			const int64_t nx = n * (n + 1);
			if (f < nx) {
				const int64_t j = f / (n + 1), fi = f % (n + 1);
				a = fi > 0 ? j * n + fi - 1 : -1;
				b = fi < n ? j * n + fi : -1;
			}
			else {
				const int64_t q = f - nx, fj = q / n, i = q % n;
				a = fj > 0 ? (fj - 1) * n + i : -1;
				b = fj < n ? fj * n + i : -1;
			}
		}
		else {
			const int64_t nx = n * n * (n + 1);
			if (f < nx) {
				const int64_t row = f / (n + 1), fi = f % (n + 1);  // row = k*n + j
				a = fi > 0 ? row * n + fi - 1 : -1;
				b = fi < n ? row * n + fi : -1;
			}
			else if (f < 2 * nx) {
				const int64_t q = f - nx, i = q % n, t = q / n, fj = t % (n + 1), k = t / (n + 1);
				a = fj > 0 ? (k * n + fj - 1) * n + i : -1;
				b = fj < n ? (k * n + fj) * n + i : -1;
			}
			else {
				const int64_t q = f - 2 * nx, i = q % n, t = q / n, j = t % n, fk = t / n;
				a = fk > 0 ? ((fk - 1) * n + j) * n + i : -1;
				b = fk < n ? (fk * n + j) * n + i : -1;
			}
		}
		double v;
		if (a >= 0 && b >= 0)
			v = -scale * (lam[a] - lam[b]) * (x[a] - x[b]);
		else {
			const int64_t c = a >= 0 ? a : b;
			v = -scale * lam[c] * x[c];
		}
		g[f] = accumulate ? g[f] + v : v;
	}
}

// dL/dA_ij = -lam_i x_j on the pattern; one thread per row
__global__ void k_value_grad(int64_t nrows, const int *__restrict__ rp, const int *__restrict__ col,
                             const double *__restrict__ lam, const double *__restrict__ x,
                             double *__restrict__ g) {
	FOR_EACH(r, nrows) {
		const double l = lam[r];
		for (int k = rp[r]; k < rp[r + 1]; ++k)
			g[k] = -l * x[col[k]];
	}
}

}  // namespace

}  // namespace fsg

using namespace fsg;

extern "C" {

FS_API int fs_fv_assemble(fs_csr Ah, int dim, int64_t n, fs_vec facesh, double scale, double shift) {
	Csr *A = reinterpret_cast<Csr *>(Ah);
	Vec *c = reinterpret_cast<Vec *>(facesh);
	if (!ok_csr(A) || !ok_vec(c))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_fv_assemble"));
	Ctx *ctx = A->ctx;
	if (dim != 2 && dim != 3)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fv_assemble: dim must be 2 or 3");
	const int64_t N = dim == 2 ? n * n : n * n * n;
	const int64_t nnz = dim == 2 ? 5 * n * n - 4 * n : 7 * n * n * n - 6 * n * n;
	const int64_t nf = dim == 2 ? 2 * n * (n + 1) : 3 * n * n * (n + 1);
	if (A->nrows != N || A->nnz != nnz || c->n != nf || c->dtype != FS_F64)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH,
		               "fs_fv_assemble: A must have the %d-D finite-volume pattern of an n^%d grid",
		               dim, dim);
	k_fv_assemble<<<grid_for(ctx, N, 256, 4), 256, 0, ctx->stream>>>(dim, n, (const double *)c->d,
	                                                               A->rowptr, A->val, scale, shift);
	FS_TRY(check_launch(ctx, "fv assemble"));
	// values changed: float copy, diagonal, CSC values and symmetric storage
	// are rebuilt on use
	invalidate_values(A);
	return FS_OK;
}

FS_API int fs_fv_face_grad(fs_ctx h, int dim, int64_t n, fs_vec lamh, fs_vec xh, double scale,
                           int accumulate, fs_vec gh) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Vec *lam = reinterpret_cast<Vec *>(lamh), *x = reinterpret_cast<Vec *>(xh),
	    *g = reinterpret_cast<Vec *>(gh);
	if (!ok_ctx(ctx) || !ok_vec(lam) || !ok_vec(x) || !ok_vec(g))
		return FS_ERR_BAD_HANDLE;
	if (dim != 2 && dim != 3)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fv_face_grad: dim must be 2 or 3");
	const int64_t N = dim == 2 ? n * n : n * n * n;
	const int64_t nf = dim == 2 ? 2 * n * (n + 1) : 3 * n * n * (n + 1);
	if (lam->n != N || x->n != N || g->n != nf || lam->dtype != FS_F64 || x->dtype != FS_F64 ||
	    g->dtype != FS_F64)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fv_face_grad: sizes do not match the grid");
	k_fv_face_grad<<<grid_for(ctx, nf, 256, 4), 256, 0, ctx->stream>>>(
		dim, n, (const double *)lam->d, (const double *)x->d, (double *)g->d, scale, accumulate);
	return check_launch(ctx, "fv face grad");
}

FS_API int fs_csr_value_grad(fs_csr Ah, fs_vec lamh, fs_vec xh, fs_vec gh) {
	Csr *A = reinterpret_cast<Csr *>(Ah);
	Vec *lam = reinterpret_cast<Vec *>(lamh), *x = reinterpret_cast<Vec *>(xh),
	    *g = reinterpret_cast<Vec *>(gh);
	if (!ok_csr(A) || !ok_vec(lam) || !ok_vec(x) || !ok_vec(g))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_value_grad"));
	if (lam->n != A->nrows || x->n != A->ncols || g->n != A->nnz || lam->dtype != FS_F64 ||
	    x->dtype != FS_F64 || g->dtype != FS_F64)
		return set_err(A->ctx, FS_ERR_SIZE_MISMATCH, "fs_csr_value_grad: sizes do not match A");
	if (A->nrows == 0)
		return FS_OK;
	k_value_grad<<<grid_for(A->ctx, A->nrows, 256, 4), 256, 0, A->ctx->stream>>>(
		A->nrows, A->rowptr, A->col, (const double *)lam->d, (const double *)x->d, (double *)g->d);
	return check_launch(A->ctx, "value grad");
}

// Materialise A^T as a new CSR matrix (the CSC view of A): the caller owns
// the result.
FS_API int fs_csr_transpose(fs_csr Ah, fs_csr *out) {
	Csr *A = reinterpret_cast<Csr *>(Ah);
	if (!ok_csr(A) || !out)
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_transpose"));
	Ctx *ctx = A->ctx;
	FS_TRY(ensure_transpose(A));
	FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // the CSC value gather
	std::vector<int> cp(A->ncols + 1), row(A->nnz);
	std::vector<double> val(A->nnz);
	FS_CUDA_TRY(ctx, cudaMemcpy(cp.data(), A->t_colptr, (A->ncols + 1) * sizeof(int), cudaMemcpyDeviceToHost));
	FS_CUDA_TRY(ctx, cudaMemcpy(row.data(), A->t_row, A->nnz * sizeof(int), cudaMemcpyDeviceToHost));
	FS_CUDA_TRY(ctx, cudaMemcpy(val.data(), A->t_val, A->nnz * sizeof(double), cudaMemcpyDeviceToHost));
	std::vector<int64_t> rp(cp.begin(), cp.end());
	return fs_csr_create(reinterpret_cast<fs_ctx>(ctx), A->ncols, A->nrows, A->nnz, rp.data(), row.data(),
	                     4, val.data(), out);
}

}  // extern "C"
