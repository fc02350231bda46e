// One color of the distributed CSR operator: flecsolve's mat::parcsr over
// topo::csr (matrices/parcsr.hh:29-177, topo/csr.hh:413-632), on this
// device.
//
// A color owns a contiguous block of rows and the column block with the same
// color (the reference's row_part / col_part, both flecsi::util::equal_map
// blocks).  Built on the host from the color's rows (global column ids), as
// the reference's coloring and init_mats build it:
//  * ghosts: the column ids outside the owned column block, sorted and
//    unique (topo/csr.hh:501-518, force_unique);
//  * diag: the owned-column entries, column = id - the block's first column
//    (cm.invert(cid).second, csr.hh:587-593);
//  * offd: the ghost entries, column = nown + the ghost's rank in the sorted
//    ghost list (the reverse colmap, csr.hh:565-569, 594-599), so offd
//    indexes the color's column vector [owned values, ghost values];
//  * both keep each row's entries in input order.
// y = diag x_own + offd x_cols, each row's two sums taken separately and
// then added (parcsr_ops::spmv, parcsr.hh:60-71: spmv_remote, spmv_local,
// y.add(y, tmp)), with the reference's row arithmetic (products rounded,
// summed left to right): the same bits as fs_parcsr_spmv of the whole
// matrix split into the same blocks.  The ghost values come from the owning
// colors: the caller's halo exchange (host-staged here) fills x_cols[nown:].
#include <algorithm>
#include <cstring>
#include <vector>

#include "fsgpu_internal.cuh"

namespace fsg {
namespace {

constexpr int kMagicPar = 0x46535058;  // 'FSPX'

struct ParCsr {
	int magic = kMagicPar;
	Ctx *ctx = nullptr;
	int64_t nrows = 0, nown = 0, col_begin = 0;
	std::vector<int64_t> colmap;  // ghost global column ids, sorted
	int64_t nnz_diag = 0, nnz_offd = 0;
	int *d_rp = nullptr, *d_col = nullptr, *o_rp = nullptr, *o_col = nullptr;
	double *d_val = nullptr, *o_val = nullptr;
};

bool ok_par(const ParCsr *p) { return p && p->magic == kMagicPar && ok_ctx(p->ctx); }

__global__ void k_parcsr_color(int n, const int *__restrict__ drp, const int *__restrict__ dcol,
                               const double *__restrict__ dval, const int *__restrict__ orp,
                               const int *__restrict__ ocol, const double *__restrict__ oval,
                               const double *__restrict__ x, double *__restrict__ y) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		// explicit roundings: a fused multiply-add would change the bits
		double yd = 0.0, yo = 0.0;
		for (int k = drp[i]; k < drp[i + 1]; ++k)
			yd = __dadd_rn(yd, __dmul_rn(dval[k], x[dcol[k]]));
		for (int k = orp[i]; k < orp[i + 1]; ++k)
			yo = __dadd_rn(yo, __dmul_rn(oval[k], x[ocol[k]]));
		y[i] = __dadd_rn(yd, yo);
	}
}

void release(ParCsr *p) {
	for (void *q : {(void *)p->d_rp, (void *)p->d_col, (void *)p->d_val, (void *)p->o_rp,
	                (void *)p->o_col, (void *)p->o_val})
		if (q)
			cudaFree(q);
}

}  // namespace
}  // namespace fsg

using namespace fsg;

extern "C" {

FS_API int fs_parcsr_create(fs_ctx h, int64_t col_begin, int64_t col_end, int64_t nrows,
                            const int64_t *rowptr, const int64_t *gcol, const double *val,
                            fs_parcsr *out) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(ctx) || !out || (nrows > 0 && !rowptr))
		return FS_ERR_BAD_HANDLE;
	*out = nullptr;
	if (nrows < 0 || col_begin < 0 || col_end < col_begin)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_parcsr_create: bad row count or column block");
	const int64_t nnz = nrows > 0 ? rowptr[nrows] : 0;
	if (nnz > 0 && (!gcol || !val))
		return set_err(ctx, FS_ERR_BAD_HANDLE, "fs_parcsr_create: missing columns or values");
	if (nnz >= ((int64_t)1 << 31) || nrows >= ((int64_t)1 << 31))
		return set_err(ctx, FS_ERR_UNSUPPORTED, "fs_parcsr_create: a color holds < 2^31 rows and entries");
	for (int64_t r = 0; r < nrows; ++r)
		if (rowptr[r + 1] < rowptr[r])
			return set_err(ctx, FS_ERR_INVALID_ARG, "fs_parcsr_create: row offsets not monotone");
	const int64_t nown = col_end - col_begin;
	auto owned = [&](int64_t c) { return c >= col_begin && c < col_end; };
	// coloring: the ghost columns, sorted and unique
	ParCsr *P = new ParCsr();
	P->ctx = ctx;
	P->nrows = nrows;
	P->nown = nown;
	P->col_begin = col_begin;
	for (int64_t k = 0; k < nnz; ++k) {
		if (gcol[k] < 0) {
			delete P;
			return set_err(ctx, FS_ERR_INVALID_ARG, "fs_parcsr_create: negative column id");
		}
		if (!owned(gcol[k]))
			P->colmap.push_back(gcol[k]);
	}
	std::sort(P->colmap.begin(), P->colmap.end());
	P->colmap.erase(std::unique(P->colmap.begin(), P->colmap.end()), P->colmap.end());
	if (nown + (int64_t)P->colmap.size() >= ((int64_t)1 << 31)) {
		delete P;
		return set_err(ctx, FS_ERR_UNSUPPORTED, "fs_parcsr_create: a color's columns exceed 2^31");
	}
	// init_mats: split every row in input order
	std::vector<int> drp(nrows + 1, 0), orp(nrows + 1, 0), dcol, ocol;
	std::vector<double> dval, oval;
	for (int64_t r = 0; r < nrows; ++r) {
		for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
			const int64_t c = gcol[k];
			if (owned(c)) {
				dcol.push_back((int)(c - col_begin));
				dval.push_back(val[k]);
			}
			else {
				const int64_t g =
					std::lower_bound(P->colmap.begin(), P->colmap.end(), c) - P->colmap.begin();
				ocol.push_back((int)(nown + g));
				oval.push_back(val[k]);
			}
		}
		drp[r + 1] = (int)dcol.size();
		orp[r + 1] = (int)ocol.size();
	}
	P->nnz_diag = (int64_t)dcol.size();
	P->nnz_offd = (int64_t)ocol.size();
	auto up = [&](void **dst, const void *src, size_t bytes) -> bool {
		if (cudaMalloc(dst, std::max<size_t>(bytes, 16)) != cudaSuccess)
			return false;
		return bytes == 0 || cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
	};
	if (!up((void **)&P->d_rp, drp.data(), drp.size() * sizeof(int)) ||
	    !up((void **)&P->o_rp, orp.data(), orp.size() * sizeof(int)) ||
	    !up((void **)&P->d_col, dcol.data(), dcol.size() * sizeof(int)) ||
	    !up((void **)&P->o_col, ocol.data(), ocol.size() * sizeof(int)) ||
	    !up((void **)&P->d_val, dval.data(), dval.size() * sizeof(double)) ||
	    !up((void **)&P->o_val, oval.data(), oval.size() * sizeof(double)) ||
	    fence_setup_copies() != cudaSuccess) {
		cudaGetLastError();
		release(P);
		delete P;
		return set_err(ctx, FS_ERR_OUT_OF_MEMORY, "fs_parcsr_create: device allocation failed");
	}
	*out = reinterpret_cast<fs_parcsr>(P);
	return FS_OK;
}

FS_API int fs_parcsr_destroy(fs_parcsr h) {
	ParCsr *P = reinterpret_cast<ParCsr *>(h);
	if (!ok_par(P))
		return FS_ERR_BAD_HANDLE;
	cudaStreamSynchronize(P->ctx->stream);
	release(P);
	P->magic = 0;
	delete P;
	return FS_OK;
}

FS_API int fs_parcsr_shape(fs_parcsr h, int64_t *nrows, int64_t *nown, int64_t *nghost,
                           int64_t *nnz_diag, int64_t *nnz_offd) {
	ParCsr *P = reinterpret_cast<ParCsr *>(h);
	if (!ok_par(P))
		return FS_ERR_BAD_HANDLE;
	if (nrows)
		*nrows = P->nrows;
	if (nown)
		*nown = P->nown;
	if (nghost)
		*nghost = (int64_t)P->colmap.size();
	if (nnz_diag)
		*nnz_diag = P->nnz_diag;
	if (nnz_offd)
		*nnz_offd = P->nnz_offd;
	return FS_OK;
}

FS_API int fs_parcsr_ghosts(fs_parcsr h, int64_t *gids, int64_t *n) {
	ParCsr *P = reinterpret_cast<ParCsr *>(h);
	if (!ok_par(P) || !n)
		return FS_ERR_BAD_HANDLE;
	const int64_t m = std::min<int64_t>(*n, (int64_t)P->colmap.size());
	if (gids && m > 0)
		memcpy(gids, P->colmap.data(), (size_t)m * sizeof(int64_t));
	*n = gids ? m : (int64_t)P->colmap.size();
	return FS_OK;
}

FS_API int fs_parcsr_color_spmv(fs_parcsr h, fs_vec xh, fs_vec yh) {
	ParCsr *P = reinterpret_cast<ParCsr *>(h);
	Vec *x = reinterpret_cast<Vec *>(xh), *y = reinterpret_cast<Vec *>(yh);
	if (!ok_par(P) || !ok_vec(x) || !ok_vec(y))
		return FS_ERR_BAD_HANDLE;
	Ctx *ctx = P->ctx;
	if (x->ctx != ctx || y->ctx != ctx || x->dtype != FS_F64 || y->dtype != FS_F64 ||
	    x->n != P->nown + (int64_t)P->colmap.size() || y->n != P->nrows)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH,
		               "fs_parcsr_color_spmv: x holds the owned then the ghost columns, y the rows");
	if (x == y)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_parcsr_color_spmv: x and y must differ");
	if (P->nrows == 0)
		return FS_OK;
	k_parcsr_color<<<grid_for(ctx, P->nrows, 256, 4), 256, 0, ctx->stream>>>(
		(int)P->nrows, P->d_rp, P->d_col, P->d_val, P->o_rp, P->o_col, P->o_val,
		(const double *)x->d, (double *)y->d);
	return check_launch(ctx, "parcsr color spmv");
}

}  // extern "C"
