// Device CSR operator: creation, row-block binning, SpMV, residual, D^-1,
// the row-block distributed (parcsr) SpMV and the CSC transpose view.
//
// Reference: mat::sparse / mat::compressed_ops (flecsolve/matrices/seq.hh:
// 35-63, 177-193), op::core::residual (operators/core.hh:129-142), the D^-1
// test operator (flecsolve/util/test/mesh.hh:123-140) and mat::parcsr
// (matrices/parcsr.hh:60-91, topo/csr.hh:413-632).
#include <algorithm>
#include <array>
#include <cstring>
#include <map>
#include <vector>

#include "spmv_kernel.cuh"

namespace fsg {

int spmv_grid(Ctx *ctx, int nblk, int per_sm) {
	int cap = ctx->sms * std::min(per_sm, 8);
	return std::max(1, std::min(nblk, cap));
}

// Row blocks of at most kBlkRows rows / kBlkNnz nonzeros; a row longer than
// kBlkNnz is a block of its own.
static std::vector<int> row_blocks(const std::vector<int> &rp) {
	const int n = (int)rp.size() - 1;
	std::vector<int> blk;
	blk.reserve(n / 64 + 2);
	blk.push_back(0);
	int r = 0;
	while (r < n) {
		const int start = r;
		if (rp[r + 1] - rp[r] > kBlkNnz) {
			r += 1;
		}
		else {
			const int base = rp[r];
			while (r < n && r - start < kBlkRows && rp[r + 1] - base <= kBlkNnz)
				++r;
		}
		blk.push_back(r);
	}
	return blk;
}

// Row patterns: the sequence of column offsets c - r of every row, numbered
// in order of first appearance.  False when a row is longer than kPatW or
// the matrix has more than kMaxPat distinct sequences; the column ids are
// used then.  Consecutive rows usually share a sequence, which is checked
// first.
static bool row_patterns(const std::vector<int> &rp, const std::vector<int> &ci,
                         std::vector<unsigned char> &pid, std::vector<int> &ptab,
                         std::vector<int> &plen, int &npat) {
	const int64_t n = (int64_t)rp.size() - 1;
	pid.assign((size_t)n + 32, 0);
	ptab.clear();
	plen.clear();
	std::map<std::array<int, kPatW + 1>, int> ids;
	std::array<int, kPatW + 1> key{}, last{};
	int last_id = -1;
	for (int64_t r = 0; r < n; ++r) {
		const int len = rp[r + 1] - rp[r];
		if (len > kPatW)
			return false;
		key.fill(0);
		key[kPatW] = len;
		for (int j = 0; j < len; ++j)
			key[j] = ci[rp[r] + j] - (int)r;
		int id;
		if (last_id >= 0 && key == last)
			id = last_id;
		else {
			auto it = ids.find(key);
			if (it == ids.end()) {
				if ((int)ids.size() == kMaxPat)
					return false;
				id = (int)ids.size();
				ids.emplace(key, id);
				ptab.insert(ptab.end(), key.begin(), key.begin() + kPatW);
				plen.push_back(len);
			}
			else
				id = it->second;
			last = key;
			last_id = id;
		}
		pid[r] = (unsigned char)id;
	}
	npat = (int)ids.size();
	return true;
}

// Per row block and 32-row warp: where the nonzeros of the warp's first row
// start, relative to the block's first nonzero (< kBlkNnz, fits a short).
static std::vector<short> warp_bases(const std::vector<int> &rp, const std::vector<int> &blk) {
	const int nblk = (int)blk.size() - 1;
	std::vector<short> wb((size_t)nblk * (kBlkRows / 32), 0);
	for (int b = 0; b < nblk; ++b)
		for (int w = 0; w < kBlkRows / 32; ++w)
			wb[(size_t)b * (kBlkRows / 32) + w] =
				(short)(rp[std::min(blk[b] + 32 * w, blk[b + 1])] - rp[blk[b]]);
	return wb;
}

// Slot codes of the symmetric storage: the positive offsets of all patterns
// (at most kMaxSym), each pattern entry coded as diagonal / upper offset k /
// lower offset k, and per pattern the entry holding each upper offset.  False
// when a negative offset has no positive partner or there are too many.
static bool sym_slots(const std::vector<int> &ptab, const std::vector<int> &plen, int npat,
                      std::vector<int> &sofs, std::vector<signed char> &pslot,
                      std::vector<signed char> &pinv) {
	sofs.clear();
	for (int p = 0; p < npat; ++p)
		for (int j = 0; j < plen[p]; ++j) {
			const int d = ptab[(size_t)p * kPatW + j];
			if (d > 0 && std::find(sofs.begin(), sofs.end(), d) == sofs.end())
				sofs.push_back(d);
		}
	if ((int)sofs.size() > kMaxSym)
		return false;
	std::sort(sofs.begin(), sofs.end());
	pslot.assign((size_t)npat * kPatW, 0);
	pinv.assign((size_t)npat * kMaxSym, -1);
	for (int p = 0; p < npat; ++p)
		for (int j = 0; j < plen[p]; ++j) {
			const int d = ptab[(size_t)p * kPatW + j];
			if (d == 0)
				continue;
			const int k = (int)(std::find(sofs.begin(), sofs.end(), d < 0 ? -d : d) - sofs.begin());
			if (k == (int)sofs.size())
				return false;
			pslot[(size_t)p * kPatW + j] = (signed char)(d > 0 ? k + 1 : -(k + 1));
			if (d > 0)
				pinv[(size_t)p * kMaxSym + k] = (signed char)j;
		}
	return true;
}

// Grid stencil: the positive offsets are 1, nx and nx ny (one, two or three
// of them) and every row r = i + nx (j + ny k) holds exactly its neighbours
// inside the nx x ny x nz grid, in column order.  Rows fall in at most 64
// boundary classes (i, j, k each at the low end, the high end or inside);
// every row of a class must carry the class's pattern.
static bool grid_dims(int64_t n, const std::vector<int> &sofs, const std::vector<unsigned char> &pid,
                      const std::vector<int> &ptab, const std::vector<int> &plen, int dims[3]) {
	const int K = (int)sofs.size();
	if (K < 1 || K > 3 || sofs[0] != 1 || n < 1)
		return false;
	int64_t nx = n, ny = 1, nz = 1;
	if (K >= 2) {
		nx = sofs[1];
		if (nx < 2 || n % nx)
			return false;
		ny = n / nx;
	}
	if (K == 3) {
		if (sofs[2] % nx || n % sofs[2])
			return false;
		ny = sofs[2] / nx;
		nz = n / sofs[2];
	}
	if (nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30))
		return false;
	const int64_t o[3] = {1, nx, nx * ny};
	int cls_pid[64];
	std::fill(cls_pid, cls_pid + 64, -1);
	int64_t r = 0;
	for (int64_t k = 0; k < nz; ++k)
		for (int64_t j = 0; j < ny; ++j)
			for (int64_t i = 0; i < nx; ++i, ++r) {
				const int64_t c[3] = {i, j, k}, e[3] = {nx, ny, nz};
				int cls = 0;
				for (int d = 0; d < 3; ++d)
					cls = cls * 4 + (c[d] == 0 ? 1 : 0) + (c[d] == e[d] - 1 ? 2 : 0);
				const int p = pid[r];
				if (cls_pid[cls] == p)
					continue;
				if (cls_pid[cls] >= 0)
					return false;
				// the class's pattern: lower neighbours from the far offset in,
				// the diagonal, upper neighbours
				int want[kPatW], len = 0;
				for (int d = K - 1; d >= 0; --d)
					if (c[d] > 0)
						want[len++] = (int)-o[d];
				want[len++] = 0;
				for (int d = 0; d < K; ++d)
					if (c[d] < e[d] - 1)
						want[len++] = (int)o[d];
				if (len != plen[p])
					return false;
				for (int q = 0; q < len; ++q)
					if (ptab[(size_t)p * kPatW + q] != want[q])
						return false;
				cls_pid[cls] = p;
			}
	dims[0] = (int)nx;
	dims[1] = (int)ny;
	dims[2] = (int)nz;
	return true;
}

static std::vector<int4> block_info(const std::vector<int> &blk, const std::vector<int> &rp) {
	std::vector<int4> info(blk.size() > 0 ? blk.size() - 1 : 0);
	for (size_t b = 0; b + 1 < blk.size(); ++b)
		info[b] = make_int4(blk[b], blk[b + 1], rp[blk[b]], rp[blk[b + 1]]);
	return info;
}

__global__ void to_f32_kernel(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x)
		b[i] = (float)a[i];
}

// dinv_i = 1 / a_ii (0 when the row has no diagonal entry, as the reference's
// D^-1 builder leaves such a value unset -> zero-initialised)
__global__ void dinv_kernel(int n, const int *__restrict__ rp, const int *__restrict__ col,
                            const double *__restrict__ val, double *__restrict__ d,
                            float *__restrict__ d32) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double v = 0.0;
		for (int k = rp[i]; k < rp[i + 1]; ++k)
			if (col[k] == i)
				v = 1.0 / val[k];
		d[i] = v;
		d32[i] = (float)v;
	}
}

int ensure_val32(Csr *A) {
	if (A->val32_valid)
		return FS_OK;
	if (A->shell_fn)
		return set_err(A->ctx, FS_ERR_UNSUPPORTED, "a shell operator has no FP32 values");
	Ctx *ctx = A->ctx;
	if (!A->val32) {
		size_t padded = (size_t)((A->nnz + 15) / 16 * 16 + 16);
		FS_CUDA_TRY(ctx, cudaMalloc(&A->val32, padded * sizeof(float)));
		FS_CUDA_TRY(ctx, cudaMemsetAsync(A->val32, 0, padded * sizeof(float), ctx->stream));
	}
	if (A->nnz > 0) {
		to_f32_kernel<<<grid_for(ctx, A->nnz, 256, 8), 256, 0, ctx->stream>>>(A->nnz, A->val, A->val32);
		FS_TRY(check_launch(ctx, "to_f32"));
	}
	A->val32_valid = true;
	return FS_OK;
}

int ensure_dinv(Csr *A) {
	if (A->dinv_valid)
		return FS_OK;
	if (A->shell_fn)
		return set_err(A->ctx, FS_ERR_INVALID_ARG, "a shell operator has no stored diagonal");
	Ctx *ctx = A->ctx;
	if (!A->dinv) {
		size_t padded = (size_t)((A->nrows + 31) / 32 * 32 + 32);
		FS_CUDA_TRY(ctx, cudaMalloc(&A->dinv, padded * sizeof(double)));
		FS_CUDA_TRY(ctx, cudaMalloc(&A->dinv32, padded * sizeof(float)));
		FS_CUDA_TRY(ctx, cudaMemsetAsync(A->dinv, 0, padded * sizeof(double), ctx->stream));
		FS_CUDA_TRY(ctx, cudaMemsetAsync(A->dinv32, 0, padded * sizeof(float), ctx->stream));
	}
	if (A->nrows > 0) {
		dinv_kernel<<<grid_for(ctx, A->nrows, 256, 4), 256, 0, ctx->stream>>>(
			(int)A->nrows, A->rowptr, A->col, A->val, A->dinv, A->dinv32);
		FS_TRY(check_launch(ctx, "dinv"));
	}
	A->dinv_valid = true;
	return FS_OK;
}

void invalidate_values(Csr *A) {
	A->values_gen++;
	A->val32_valid = false;
	A->dinv_valid = false;
	A->t_vals_valid = false;
	A->sym64_valid = false;
	A->sym32_valid = false;
	A->gen64_valid = false;
	A->gen32_valid = false;
	A->sym_state = -1;
}

// The diagonal and upper diagonals from the CSR values, and the check that
// every lower entry a(r, r - d) equals its partner a(r - d, r) bit for bit
// (else *bad is set and the storage is not used).
template<class V>
__global__ void k_sym_build(int n, const int *__restrict__ rp, const double *__restrict__ val,
                            const unsigned char *__restrict__ pid,
                            const unsigned char *__restrict__ plen,
                            const signed char *__restrict__ pslot,
                            const signed char *__restrict__ pinv, const int *__restrict__ sofs,
                            int64_t ld, V *__restrict__ diag, V *__restrict__ up, int check,
                            unsigned *bad) {
	for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
		const int p = pid[r], len = plen[p], k0 = rp[r];
		for (int j = 0; j < len; ++j) {
			const int code = pslot[p * kPatW + j];
			const double v = val[k0 + j];
			if (code == 0)
				diag[r] = (V)v;
			else if (code > 0)
				up[(int64_t)(code - 1) * ld + r] = (V)v;
			else if (check) {
				const int k = -code - 1, c = r - sofs[k];
				const int jj = c >= 0 ? pinv[pid[c] * kMaxSym + k] : -1;
				if (jj < 0 || __double_as_longlong(val[rp[c] + jj]) != __double_as_longlong(v))
					atomicOr(bad, 1u);
			}
		}
	}
}

// The general grid storage of a grid stencil with asymmetric values: every
// entry of row r at row r of its array (diagonal, upper diagonal d at
// (1 + d) ld, lower diagonal d at (1 + nsym + d) ld, d = 0 .. nsym - 1).
template<class V>
__global__ void k_gen_build(int n, const int *__restrict__ rp, const double *__restrict__ val,
                            const unsigned char *__restrict__ pid,
                            const unsigned char *__restrict__ plen,
                            const signed char *__restrict__ pslot, int nsym, int64_t ld,
                            V *__restrict__ S) {
	for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
		const int p = pid[r], len = plen[p], k0 = rp[r];
		for (int j = 0; j < len; ++j) {
			const int code = pslot[p * kPatW + j];
			const int64_t slot = code >= 0 ? code : nsym - code;  // 0, 1..nsym, nsym+1..2 nsym
			S[slot * ld + r] = (V)val[k0 + j];
		}
	}
}

static int ensure_gen(Csr *A, bool f32) {
	if (A->coding != kCodingGrid || A->grid_nx <= 0 || A->grid_nx % 4 || A->sym_state != 0)
		return FS_OK;
	bool &valid = f32 ? A->gen32_valid : A->gen64_valid;
	if (valid)
		return FS_OK;
	Ctx *ctx = A->ctx;
	const size_t elems = (size_t)(2 * A->nsym + 1) * (size_t)A->sym_ld;
	void **buf = f32 ? (void **)&A->gen32 : (void **)&A->gen64;
	if (!*buf) {
		const size_t bytes = elems * (f32 ? sizeof(float) : sizeof(double));
		FS_CUDA_TRY(ctx, cudaMalloc(buf, bytes));
		FS_CUDA_TRY(ctx, cudaMemsetAsync(*buf, 0, bytes, ctx->stream));
	}
	const int n = (int)A->nrows;
	if (f32)
		k_gen_build<float><<<grid_for(ctx, n, 256, 4), 256, 0, ctx->stream>>>(
			n, A->rowptr, A->val, A->pid, A->plen, A->pslot, A->nsym, A->sym_ld, A->gen32);
	else
		k_gen_build<double><<<grid_for(ctx, n, 256, 4), 256, 0, ctx->stream>>>(
			n, A->rowptr, A->val, A->pid, A->plen, A->pslot, A->nsym, A->sym_ld, A->gen64);
	FS_TRY(check_launch(ctx, "general grid storage"));
	valid = true;
	return FS_OK;
}

int ensure_sym(Csr *A, bool f32) {
	if (!A->pslot || A->coding < kCodingSym)
		return FS_OK;
	if (A->sym_state == 0)
		return ensure_gen(A, f32);
	bool &valid = f32 ? A->sym32_valid : A->sym64_valid;
	if (valid)
		return FS_OK;
	Ctx *ctx = A->ctx;
	const size_t elems = (size_t)(A->nsym + 1) * (size_t)A->sym_ld;
	void **buf = f32 ? (void **)&A->sym32 : (void **)&A->sym64;
	if (!*buf) {
		const size_t bytes = elems * (f32 ? sizeof(float) : sizeof(double));
		FS_CUDA_TRY(ctx, cudaMalloc(buf, bytes));
		FS_CUDA_TRY(ctx, cudaMemsetAsync(*buf, 0, bytes, ctx->stream));
	}
	if (!A->sym_flag)
		FS_CUDA_TRY(ctx, cudaMalloc(&A->sym_flag, sizeof(unsigned)));
	const int check = A->sym_state < 0;
	if (check)
		FS_CUDA_TRY(ctx, cudaMemsetAsync(A->sym_flag, 0, sizeof(unsigned), ctx->stream));
	const int n = (int)A->nrows;
	if (f32)
		k_sym_build<float><<<grid_for(ctx, n, 256, 4), 256, 0, ctx->stream>>>(
			n, A->rowptr, A->val, A->pid, A->plen, A->pslot, A->pinv, A->sofs, A->sym_ld, A->sym32,
			A->sym32 + A->sym_ld, check, A->sym_flag);
	else
		k_sym_build<double><<<grid_for(ctx, n, 256, 4), 256, 0, ctx->stream>>>(
			n, A->rowptr, A->val, A->pid, A->plen, A->pslot, A->pinv, A->sofs, A->sym_ld, A->sym64,
			A->sym64 + A->sym_ld, check, A->sym_flag);
	FS_TRY(check_launch(ctx, "symmetric storage"));
	if (check) {
		unsigned bad = 0;
		FS_CUDA_TRY(ctx, cudaMemcpyAsync(&bad, A->sym_flag, sizeof(unsigned), cudaMemcpyDeviceToHost,
		                                 ctx->stream));
		FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
		A->sym_state = bad ? 0 : 1;
	}
	valid = A->sym_state == 1;
	if (A->sym_state == 0)
		return ensure_gen(A, f32);
	return FS_OK;
}

// ------------------------------------------------------ parcsr split --

// y_i = (sum over owned columns) + (sum over ghost columns), each summed in
// CSR order.  Row blocks as flecsi::util::equal_map makes them (FleCSI 2.4,
// flecsi/util/color_map.hh, restated): blocks of q = n / P rows, the first
// r = n % P one row longer; row i is in block i / (q + 1) below (q + 1) r and
// in block r + (i - (q + 1) r) / q above.
template<bool EXACT>
__global__ void parcsr_kernel(int n, int parts, const int *__restrict__ rp,
                              const int *__restrict__ col, const double *__restrict__ val,
                              const double *__restrict__ x, double *__restrict__ y) {
	const int q = n / parts, rem = n % parts;
	const int brk = (q + 1) * rem;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const int c = i < brk ? i / (q + 1) : rem + (i - brk) / q;
		const int lo = c * q + (c < rem ? c : rem);
		const int hi = lo + q + (c < rem ? 1 : 0);
		double yd = 0.0, yo = 0.0;
		for (int k = rp[i]; k < rp[i + 1]; ++k) {
			const int j = col[k];
			if (EXACT) {
				// explicit roundings: nvcc would otherwise contract the
				// product and the sum into one fused multiply-add
				double p = __dmul_rn(val[k], x[j]);
				if (j >= lo && j < hi)
					yd = __dadd_rn(yd, p);
				else
					yo = __dadd_rn(yo, p);
			}
			else {
				if (j >= lo && j < hi)
					yd = fma(val[k], x[j], yd);
				else
					yo = fma(val[k], x[j], yo);
			}
		}
		y[i] = __dadd_rn(yd, yo);
	}
}

// ------------------------------------------------- transpose (CSC) view --

// counting sort of the CSR entries by column, stable in row order, built on
// the host once per pattern; values gathered through the permutation
__global__ void gather_kernel(int64_t n, const int *__restrict__ perm,
                              const double *__restrict__ src, double *__restrict__ dst) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x)
		dst[i] = src[perm[i]];
}

int ensure_transpose(Csr *A) {
	Ctx *ctx = A->ctx;
	FS_TRY(reject_matrix_free(A, "transpose"));
	if (!A->t_valid) {
		const int64_t n = A->nrows, m = A->ncols, nnz = A->nnz;
		std::vector<int> hcol(nnz);
		FS_CUDA_TRY(ctx, cudaMemcpy(hcol.data(), A->col, nnz * sizeof(int), cudaMemcpyDeviceToHost));
		std::vector<int> cp(m + 1, 0), trow(nnz), perm(nnz);
		for (int64_t k = 0; k < nnz; ++k)
			cp[hcol[k] + 1]++;
		for (int64_t j = 0; j < m; ++j)
			cp[j + 1] += cp[j];
		std::vector<int> fill(cp.begin(), cp.end() - 1);
		for (int64_t i = 0; i < n; ++i)
			for (int k = A->h_rowptr[i]; k < A->h_rowptr[i + 1]; ++k) {
				int slot = fill[hcol[k]]++;
				trow[slot] = (int)i;
				perm[slot] = k;
			}
		std::vector<int> tb = row_blocks(cp);
		std::vector<int4> tinfo = block_info(tb, cp);
		size_t padded = (size_t)((nnz + 15) / 16 * 16 + 16);
		FS_CUDA_TRY(ctx, cudaMalloc(&A->t_colptr, (m + 1 + 16) * sizeof(int)));
		FS_CUDA_TRY(ctx, cudaMemset(A->t_colptr, 0, (m + 1 + 16) * sizeof(int)));
		FS_CUDA_TRY(ctx, cudaMalloc(&A->t_row, padded * sizeof(int)));
		FS_CUDA_TRY(ctx, cudaMalloc(&A->t_perm, padded * sizeof(int)));
		FS_CUDA_TRY(ctx, cudaMalloc(&A->t_val, padded * sizeof(double)));
		FS_CUDA_TRY(ctx, cudaMalloc(&A->t_blk, tb.size() * sizeof(int)));
		FS_CUDA_TRY(ctx, cudaMalloc(&A->t_blkinfo, std::max<size_t>(1, tinfo.size()) * sizeof(int4)));
		if (!tinfo.empty())
			FS_CUDA_TRY(ctx, cudaMemcpy(A->t_blkinfo, tinfo.data(), tinfo.size() * sizeof(int4),
			                            cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, cudaMemset(A->t_row, 0, padded * sizeof(int)));
		FS_CUDA_TRY(ctx, cudaMemset(A->t_val, 0, padded * sizeof(double)));
		FS_CUDA_TRY(ctx, cudaMemcpy(A->t_colptr, cp.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, cudaMemcpy(A->t_row, trow.data(), nnz * sizeof(int), cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, cudaMemcpy(A->t_perm, perm.data(), nnz * sizeof(int), cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, cudaMemcpy(A->t_blk, tb.data(), tb.size() * sizeof(int), cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, fence_setup_copies());
		A->t_nblk = (int)tb.size() - 1;
		A->t_valid = true;
		A->t_vals_valid = false;
	}
	if (!A->t_vals_valid) {
		if (A->nnz > 0) {
			gather_kernel<<<grid_for(ctx, A->nnz, 256, 8), 256, 0, ctx->stream>>>(
				A->nnz, A->t_perm, A->val, A->t_val);
			FS_TRY(check_launch(ctx, "csc gather"));
		}
		A->t_vals_valid = true;
	}
	return FS_OK;
}

int transpose_spmv(Csr *A, const double *x, double *y) {
	FS_TRY(ensure_transpose(A));
	Csr T;  // a view sharing the CSC arrays
	T.ctx = A->ctx;
	T.view = true;
	T.nrows = A->ncols;
	T.ncols = A->nrows;
	T.nnz = A->nnz;
	T.rowptr = A->t_colptr;
	T.col = A->t_row;
	T.val = A->t_val;
	T.blk = A->t_blk;
	T.blkinfo = A->t_blkinfo;
	T.nblk = A->t_nblk;
	int st = launch_spmv<double, false, false>(A->ctx, &T, A->t_val, x, nullptr,
	                                           EpiStore<double>{y});
	T.magic = 0;
	T.rowptr = nullptr;
	T.col = nullptr;
	T.val = nullptr;
	T.blk = nullptr;
	T.blkinfo = nullptr;
	return st;
}

// y = A x through the caller's callback.  The context's stream is drained
// first, so x is complete whichever stream or host code the callback reads it
// from; the callback returns once y is written or its writes are enqueued on
// the context's stream.
int shell_apply(const Csr *A, Vec *x, Vec *y) {
	Ctx *ctx = A->ctx;
	if (x->dtype != FS_F64 || y->dtype != FS_F64)
		return set_err(ctx, FS_ERR_UNSUPPORTED, "a shell operator applies to FP64 vectors");
	if (x->n != A->ncols || y->n != A->nrows)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "shell operator: vector sizes do not match");
	FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	const int rc = A->shell_fn(A->shell_user, reinterpret_cast<fs_vec>(x), reinterpret_cast<fs_vec>(y));
	if (rc != 0)
		return set_err(ctx, FS_ERR_CALLBACK, "shell operator callback returned %d", rc);
	return FS_OK;
}

// ------------------------------------------------ vector-SpMV tuning --

// lanes per row from the mean row length (0: the row-block kernel)
static int lanes_from_mean(const Csr *A) {
	const double mean = A->nrows > 0 ? (double)A->nnz / (double)A->nrows : 0.0;
	if (mean < 16.0)
		return 0;
	return mean < 32.0 ? 4 : mean < 64.0 ? 8 : mean < 128.0 ? 16 : 32;
}

// mean time of `reps` FMA-mode SpMVs y = A x with `lanes` (0: row blocks)
template<class V>
static int time_lanes(Ctx *ctx, const Csr *A, const V *vals, const V *x, V *y, int lanes,
                      float *ms) {
	auto once = [&]() -> int {
		if (lanes > 0)
			return launch_spmv_vec<V, false>(ctx, A, vals, x, (const V *)nullptr, EpiStore<V>{y},
			                                 lanes);
		CsrDev<V> d{A->rowptr, A->col, vals, A->blkinfo, A->nblk, ctx->dev_err};
		return launch_spmv_as<V, false, false>(ctx, d, x, (const V *)nullptr, EpiStore<V>{y});
	};
	constexpr int reps = 5;
	FS_TRY(once());
	FS_TRY(once());
	cudaEvent_t e0, e1;
	if (cudaEventCreate(&e0) != cudaSuccess)
		return set_err(ctx, FS_ERR_CUDA, "spmv tuning: event creation failed");
	if (cudaEventCreate(&e1) != cudaSuccess) {
		cudaEventDestroy(e0);
		return set_err(ctx, FS_ERR_CUDA, "spmv tuning: event creation failed");
	}
	int rc = cudaEventRecord(e0, ctx->stream) == cudaSuccess ? FS_OK : FS_ERR_CUDA;
	for (int i = 0; i < reps && rc == FS_OK; ++i)
		rc = once();
	if (rc == FS_OK && (cudaEventRecord(e1, ctx->stream) != cudaSuccess ||
	                    cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(ms, e0, e1) != cudaSuccess))
		rc = set_err(ctx, FS_ERR_CUDA, "spmv tuning: timing failed");
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

// The binned schedule of the vector SpMV: rows by length class (<= 8, <= 32,
// <= 128 nonzeros, longer: 4, 8, 16, 32 lanes), longest class first, each
// class in row order, cut into warp tasks of 32 / lanes rows
static int ensure_bins(Csr *A) {
	if (A->bin_task || A->nrows == 0)
		return FS_OK;
	const std::vector<int> &rp = A->h_rowptr;
	if ((int64_t)rp.size() != A->nrows + 1)
		return set_err(A->ctx, FS_ERR_INVALID_ARG, "spmv: no host row offsets for the binned schedule");
	std::vector<int> cls[4];
	for (int64_t r = 0; r < A->nrows; ++r) {
		const int len = rp[r + 1] - rp[r];
		cls[len <= 8 ? 0 : len <= 32 ? 1 : len <= 128 ? 2 : 3].push_back((int)r);
	}
	std::vector<int> rows;
	std::vector<int2> task;
	rows.reserve(A->nrows);
	for (int c = 3; c >= 0; --c) {
		const int L = 4 << c, per = 32 / L;
		const int base = (int)rows.size();
		for (size_t i = 0; i < cls[c].size(); i += per)
			task.push_back(make_int2(base + (int)i, L | (int)(std::min<size_t>(per, cls[c].size() - i) << 8)));
		rows.insert(rows.end(), cls[c].begin(), cls[c].end());
	}
	if (cudaMalloc(&A->bin_rows, rows.size() * sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&A->bin_task, task.size() * sizeof(int2)) != cudaSuccess ||
	    cudaMemcpy(A->bin_rows, rows.data(), rows.size() * sizeof(int), cudaMemcpyHostToDevice) !=
	        cudaSuccess ||
	    cudaMemcpy(A->bin_task, task.data(), task.size() * sizeof(int2), cudaMemcpyHostToDevice) !=
	        cudaSuccess ||
	    fence_setup_copies() != cudaSuccess) {
		cudaGetLastError();
		cudaFree(A->bin_rows);
		cudaFree(A->bin_task);
		A->bin_rows = nullptr;
		A->bin_task = nullptr;
		return set_err(A->ctx, FS_ERR_OUT_OF_MEMORY, "spmv: binned schedule allocation failed");
	}
	A->bin_ntask = (int)task.size();
	return FS_OK;
}

// Time the row-block kernel, the vector kernel with 4, 8, 16 and 32 lanes
// per row and the binned vector kernel on A's values of one type; *best =
// the fastest
static int tune_lanes(Ctx *ctx, Csr *A, bool f32, int *best) {
	if (f32)
		FS_TRY(ensure_val32(A));
	FS_TRY(ensure_bins(A));
	const size_t vb = f32 ? 4 : 8;
	void *x = nullptr, *y = nullptr;
	if (cudaMalloc(&x, (size_t)(A->ncols + 32) * vb) != cudaSuccess ||
	    cudaMalloc(&y, (size_t)(A->nrows + 32) * vb) != cudaSuccess) {
		cudaGetLastError();
		if (x)
			cudaFree(x);
		return set_err(ctx, FS_ERR_OUT_OF_MEMORY, "spmv tuning: scratch allocation failed");
	}
	int rc = cudaMemsetAsync(x, 0, (size_t)(A->ncols + 32) * vb, ctx->stream) == cudaSuccess
	             ? FS_OK
	             : FS_ERR_CUDA;
	float best_ms = 0.f;
	*best = 0;
	for (int lanes : {0, 4, 8, 16, 32, 1}) {
		if (rc != FS_OK)
			break;
		float ms = 0.f;
		rc = f32 ? time_lanes<float>(ctx, A, A->val32, (const float *)x, (float *)y, lanes, &ms)
		         : time_lanes<double>(ctx, A, A->val, (const double *)x, (double *)y, lanes, &ms);
		if (rc == FS_OK && (lanes == 0 || ms < best_ms)) {
			best_ms = ms;
			*best = lanes;
		}
	}
	cudaStreamSynchronize(ctx->stream);
	cudaFree(x);
	cudaFree(y);
	return rc;
}

int spmv_lanes(Ctx *ctx, const Csr *A, bool f32) {
	// stencil operators keep the row formats (all of them give the same bits)
	if (A->pid || A->nrows == 0 || stores_no_rows(A))
		return 0;
	if (A->view)
		return lanes_from_mean(A);
	Csr *M = const_cast<Csr *>(A);
	int &lanes = M->vec_lanes[f32 ? 1 : 0];
	if (lanes >= 0)
		return lanes;
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
		cudaGetLastError();
		return lanes_from_mean(A);
	}
	int best = 0;
	if (tune_lanes(ctx, M, f32, &best) != FS_OK) {
		cudaGetLastError();
		best = lanes_from_mean(A);
	}
	lanes = best;
	return lanes;
}

}  // namespace fsg

using namespace fsg;

extern "C" {

FS_API int fs_csr_tune(fs_csr h, int dtype, int *lanes) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_tune"));
	if (dtype != FS_F64 && dtype != FS_F32)
		return set_err(A->ctx, FS_ERR_INVALID_ARG, "fs_csr_tune: dtype must be FS_F64 or FS_F32");
	const bool f32 = dtype == FS_F32;
	int best = 0;
	if (!A->pid && A->nrows > 0) {
		FS_TRY(tune_lanes(A->ctx, A, f32, &best));
		A->vec_lanes[f32 ? 1 : 0] = best;
	}
	if (lanes)
		*lanes = best;
	return FS_OK;
}

FS_API int fs_csr_set_lanes(fs_csr h, int dtype, int lanes) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_set_lanes"));
	if (dtype != FS_F64 && dtype != FS_F32)
		return set_err(A->ctx, FS_ERR_INVALID_ARG, "fs_csr_set_lanes: dtype must be FS_F64 or FS_F32");
	if (lanes != -1 && lanes != 0 && lanes != 1 && lanes != 4 && lanes != 8 && lanes != 16 &&
	    lanes != 32)
		return set_err(A->ctx, FS_ERR_INVALID_ARG,
		               "fs_csr_set_lanes: lanes must be -1, 0, 1, 4, 8, 16 or 32");
	if (lanes == 1 && !A->pid)
		FS_TRY(ensure_bins(A));
	A->vec_lanes[dtype == FS_F32 ? 1 : 0] = lanes;
	return FS_OK;
}

FS_API int fs_csr_create(fs_ctx h, int64_t nrows, int64_t ncols, int64_t nnz,
                         const int64_t *rowptr, const void *col, int index_bytes,
                         const double *val, fs_csr *out) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(ctx) || !out)
		return FS_ERR_BAD_HANDLE;
	*out = nullptr;
	if (nrows < 0 || ncols < 0 || nnz < 0 || !rowptr || (nnz > 0 && (!col || !val)))
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_create: bad arguments");
	if (index_bytes != 4 && index_bytes != 8)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_create: index_bytes must be 4 or 8");
	if (nnz >= (int64_t)1 << 31 || nrows >= (int64_t)1 << 31 || ncols >= (int64_t)1 << 31)
		return set_err(ctx, FS_ERR_UNSUPPORTED,
		               "fs_csr_create: the library stores 32-bit offsets (nnz, rows < 2^31)");
	if (rowptr[0] != 0 || rowptr[nrows] != nnz)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_create: rowptr[0] must be 0 and rowptr[n] = nnz");
	std::vector<int> rp(nrows + 1);
	for (int64_t i = 0; i <= nrows; ++i) {
		if (i > 0 && rowptr[i] < rowptr[i - 1])
			return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_create: rowptr not monotone at %lld", (long long)i);
		rp[i] = (int)rowptr[i];
	}
	size_t padded = (size_t)((nnz + 15) / 16 * 16 + 16);
	std::vector<int> ci(padded, 0);
	for (int64_t k = 0; k < nnz; ++k) {
		int64_t c = index_bytes == 4 ? (int64_t)((const int32_t *)col)[k] : ((const int64_t *)col)[k];
		if (c < 0 || c >= ncols)
			return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_create: column %lld out of range at %lld",
			               (long long)c, (long long)k);
		ci[k] = (int)c;
	}
	std::vector<int> blk = row_blocks(rp);
	std::vector<int4> binfo = block_info(blk, rp);

	Csr *A = new Csr();
	A->ctx = ctx;
	A->nrows = nrows;
	A->ncols = ncols;
	A->nnz = nnz;
	A->nblk = (int)blk.size() - 1;
	A->h_rowptr = rp;
	auto fail = [&](int st) {
		cudaFree(A->rowptr);
		cudaFree(A->col);
		cudaFree(A->val);
		cudaFree(A->blk);
		cudaFree(A->blkinfo);
		delete A;
		cudaGetLastError();
		return set_err(ctx, st, "fs_csr_create: device allocation or copy failed");
	};
	if (cudaMalloc(&A->rowptr, (nrows + 1 + 16) * sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&A->col, padded * sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&A->val, padded * sizeof(double)) != cudaSuccess ||
	    cudaMalloc(&A->blk, blk.size() * sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&A->blkinfo, std::max<size_t>(1, binfo.size()) * sizeof(int4)) != cudaSuccess)
		return fail(FS_ERR_OUT_OF_MEMORY);
	if (cudaMemset(A->rowptr, 0, (nrows + 1 + 16) * sizeof(int)) != cudaSuccess ||
	    cudaMemcpy(A->rowptr, rp.data(), (nrows + 1) * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(A->col, ci.data(), padded * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemset(A->val, 0, padded * sizeof(double)) != cudaSuccess ||
	    (nnz > 0 && cudaMemcpy(A->val, val, nnz * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) ||
	    cudaMemcpy(A->blk, blk.data(), blk.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
	    (!binfo.empty() && cudaMemcpy(A->blkinfo, binfo.data(), binfo.size() * sizeof(int4),
	                                  cudaMemcpyHostToDevice) != cudaSuccess) ||
	    fence_setup_copies() != cudaSuccess)
		return fail(FS_ERR_CUDA);
	std::vector<unsigned char> pid;
	std::vector<int> ptab, plen;
	int npat = 0;
	if (nnz > 0 && nrows > 0 && row_patterns(rp, ci, pid, ptab, plen, npat)) {
		if (cudaMalloc(&A->pid, pid.size()) != cudaSuccess ||
		    cudaMalloc(&A->ptab, ptab.size() * sizeof(int)) != cudaSuccess ||
		    cudaMemcpy(A->pid, pid.data(), pid.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		    cudaMemcpy(A->ptab, ptab.data(), ptab.size() * sizeof(int), cudaMemcpyHostToDevice) !=
		        cudaSuccess ||
		    fence_setup_copies() != cudaSuccess) {
			cudaFree(A->pid);
			cudaFree(A->ptab);
			return fail(FS_ERR_OUT_OF_MEMORY);
		}
		A->npat = npat;
		std::vector<short> wb = warp_bases(rp, blk);
		std::vector<unsigned char> pl(plen.begin(), plen.end());
		pl.resize(std::max<size_t>(pl.size(), 16), 0);
		if (cudaMalloc(&A->pwb, wb.size() * sizeof(short)) != cudaSuccess ||
		    cudaMalloc(&A->plen, pl.size()) != cudaSuccess ||
		    cudaMemcpy(A->pwb, wb.data(), wb.size() * sizeof(short), cudaMemcpyHostToDevice) !=
		        cudaSuccess ||
		    cudaMemcpy(A->plen, pl.data(), pl.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
		    fence_setup_copies() != cudaSuccess) {
			cudaFree(A->pid);
			cudaFree(A->ptab);
			cudaFree(A->pwb);
			cudaFree(A->plen);
			return fail(FS_ERR_OUT_OF_MEMORY);
		}
		std::vector<int> sofs;
		std::vector<signed char> pslot, pinv;
		const int64_t sym_ld = (nrows + 31) / 32 * 32 + 32;
		if (nrows == ncols && sym_slots(ptab, plen, npat, sofs, pslot, pinv) &&
		    (int64_t)(sofs.size() + 1) * sym_ld < ((int64_t)1 << 31)) {
			// per pattern entry: value at S[r + vo], column r + xo (S holds the
			// diagonal, then upper diagonal k at (k + 1) * ld)
			std::vector<int2> stab((size_t)npat * kPatW, make_int2(0, 0));
			for (int p = 0; p < npat; ++p)
				for (int j = 0; j < plen[p]; ++j) {
					const int code = pslot[(size_t)p * kPatW + j];
					const int d = ptab[(size_t)p * kPatW + j];
					int vo = 0;
					if (code > 0)
						vo = (int)(code * sym_ld);
					else if (code < 0)
						vo = (int)(-code * sym_ld) + d;  // d < 0: u at r + d
					stab[(size_t)p * kPatW + j] = make_int2(vo, d);
				}
			if (cudaMalloc(&A->stab, stab.size() * sizeof(int2)) != cudaSuccess ||
			    cudaMemcpy(A->stab, stab.data(), stab.size() * sizeof(int2), cudaMemcpyHostToDevice) !=
			        cudaSuccess ||
			    cudaMalloc(&A->pslot, pslot.size()) != cudaSuccess ||
			    cudaMalloc(&A->pinv, pinv.size()) != cudaSuccess ||
			    cudaMalloc(&A->sofs, std::max<size_t>(1, sofs.size()) * sizeof(int)) != cudaSuccess ||
			    cudaMemcpy(A->pslot, pslot.data(), pslot.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
			    cudaMemcpy(A->pinv, pinv.data(), pinv.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
			    (!sofs.empty() && cudaMemcpy(A->sofs, sofs.data(), sofs.size() * sizeof(int),
			                                 cudaMemcpyHostToDevice) != cudaSuccess) ||
			    fence_setup_copies() != cudaSuccess) {
				for (void *q : {(void *)A->pid, (void *)A->ptab, (void *)A->pwb, (void *)A->plen, (void *)A->pslot, (void *)A->pinv,
	                (void *)A->sofs, (void *)A->stab, (void *)A->sym64, (void *)A->sym32, (void *)A->sym_flag,
				                (void *)A->pslot, (void *)A->pinv, (void *)A->sofs})
					cudaFree(q);
				return fail(FS_ERR_OUT_OF_MEMORY);
			}
			A->nsym = (int)sofs.size();
			A->sym_ld = sym_ld;
			int dims[3];
			if (grid_dims(nrows, sofs, pid, ptab, plen, dims)) {
				A->grid_nx = dims[0];
				A->grid_ny = dims[1];
				A->grid_nz = dims[2];
			}
		}
	}
	*out = reinterpret_cast<fs_csr>(A);
	return FS_OK;
}

FS_API int fs_csr_index_coding(fs_csr h, int enable, int *active) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_index_coding"));
	if (enable > kCodingGrid)
		return set_err(A->ctx, FS_ERR_INVALID_ARG,
		               "fs_csr_index_coding: enable must be -1, 0, 1, 2 or 3");
	if (enable >= 0)
		A->coding = enable;
	if (active) {
		FS_TRY(ensure_sym(A, false));
		*active = active_coding(A);
	}
	return FS_OK;
}

FS_API int fs_csr_grid_dims(fs_csr h, int64_t dims[3]) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A) || !dims)
		return FS_ERR_BAD_HANDLE;
	dims[0] = A->grid_nx;
	dims[1] = A->grid_ny;
	dims[2] = A->grid_nz;
	return FS_OK;
}

FS_API int fs_csr_row_blocks(fs_csr h, int64_t *nblk) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A) || !nblk)
		return FS_ERR_BAD_HANDLE;
	*nblk = A->nblk;
	return FS_OK;
}

FS_API int fs_shell_create(fs_ctx h, int64_t nrows, int64_t ncols, fs_op_fn fn, void *user,
                           fs_csr *out) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(ctx) || !out)
		return FS_ERR_BAD_HANDLE;
	*out = nullptr;
	if (!fn || nrows < 0 || ncols < 0)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_shell_create: a callback and sizes >= 0 are required");
	Csr *A = new Csr();
	A->ctx = ctx;
	A->nrows = nrows;
	A->ncols = ncols;
	A->shell_fn = fn;
	A->shell_user = user;
	*out = reinterpret_cast<fs_csr>(A);
	return FS_OK;
}

FS_API int fs_csr_destroy(fs_csr h) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	cudaStreamSynchronize(A->ctx->stream);
	destroy_batch_plans(A);
	for (void *p : {(void *)A->rowptr, (void *)A->col, (void *)A->val, (void *)A->val32,
	                (void *)A->blk, (void *)A->blkinfo, (void *)A->dinv, (void *)A->dinv32,
	                (void *)A->pid, (void *)A->ptab, (void *)A->pwb, (void *)A->plen, (void *)A->pslot, (void *)A->pinv,
	                (void *)A->sofs, (void *)A->stab, (void *)A->sym64, (void *)A->sym32, (void *)A->sym_flag,
	                (void *)A->t_colptr, (void *)A->t_row, (void *)A->t_perm, (void *)A->t_val,
	                (void *)A->t_blk, (void *)A->t_blkinfo, (void *)A->bin_rows, (void *)A->bin_task,
	                (void *)A->gen64, (void *)A->gen32})
		if (p)
			cudaFree(p);
	destroy_fvm(A->fvm);
	A->magic = 0;
	delete A;
	return FS_OK;
}

FS_API int fs_csr_shape(fs_csr h, int64_t *nrows, int64_t *ncols, int64_t *nnz) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	if (nrows) *nrows = A->nrows;
	if (ncols) *ncols = A->ncols;
	if (nnz) *nnz = A->nnz;
	return FS_OK;
}

FS_API int fs_csr_update_values(fs_csr h, const double *val) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_update_values"));
	if (A->nnz > 0 && !val)
		return FS_ERR_INVALID_ARG;
	if (A->nnz > 0)
		FS_CUDA_TRY(A->ctx, cudaMemcpyAsync(A->val, val, A->nnz * sizeof(double),
		                                    cudaMemcpyHostToDevice, A->ctx->stream));
	FS_CUDA_TRY(A->ctx, cudaStreamSynchronize(A->ctx->stream));
	invalidate_values(A);
	return FS_OK;
}

FS_API int fs_csr_update_values_device(fs_csr h, const double *dval) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_update_values_device"));
	if (A->nnz > 0 && !dval)
		return FS_ERR_INVALID_ARG;
	if (A->nnz > 0 && dval != A->val)
		FS_CUDA_TRY(A->ctx, cudaMemcpyAsync(A->val, dval, A->nnz * sizeof(double),
		                                    cudaMemcpyDeviceToDevice, A->ctx->stream));
	invalidate_values(A);
	return FS_OK;
}

FS_API int fs_csr_values_device_ptr(fs_csr h, double **dval) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A) || !dval)
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_values_device_ptr"));
	*dval = A->val;
	// the caller may write through the pointer: derived data is rebuilt
	invalidate_values(A);
	return FS_OK;
}

FS_API int fs_csr_spmv(fs_csr h, fs_vec xh, fs_vec yh, int mode) {
	Csr *A = reinterpret_cast<Csr *>(h);
	Vec *x = reinterpret_cast<Vec *>(xh), *y = reinterpret_cast<Vec *>(yh);
	if (!ok_csr(A) || !ok_vec(x) || !ok_vec(y))
		return FS_ERR_BAD_HANDLE;
	Ctx *ctx = A->ctx;
	if (x->n != A->ncols || y->n != A->nrows || x->dtype != y->dtype)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_csr_spmv: shapes/dtypes do not match");
	if (x == y)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_spmv: x and y must differ");
	if (mode != FS_SPMV_FMA && mode != FS_SPMV_EXACT)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_spmv: bad mode");
	if (A->shell_fn)
		return shell_apply(A, x, y);
	if (A->nrows == 0)
		return FS_OK;
	FS_TRY(ensure_sym(A, x->dtype == FS_F32));
	if (x->dtype == FS_F64) {
		EpiStore<double> e{(double *)y->d};
		if (mode == FS_SPMV_EXACT)
			return launch_spmv<double, true, false>(ctx, A, A->val, (const double *)x->d, nullptr, e);
		return launch_spmv<double, false, false>(ctx, A, A->val, (const double *)x->d, nullptr, e);
	}
	FS_TRY(ensure_val32(A));
	EpiStore<float> e{(float *)y->d};
	if (mode == FS_SPMV_EXACT)
		return launch_spmv<float, true, false>(ctx, A, A->val32, (const float *)x->d, nullptr, e);
	return launch_spmv<float, false, false>(ctx, A, A->val32, (const float *)x->d, nullptr, e);
}

FS_API int fs_csr_residual(fs_csr h, fs_vec bh, fs_vec xh, fs_vec rh) {
	Csr *A = reinterpret_cast<Csr *>(h);
	Vec *b = reinterpret_cast<Vec *>(bh), *x = reinterpret_cast<Vec *>(xh),
	    *r = reinterpret_cast<Vec *>(rh);
	if (!ok_csr(A) || !ok_vec(b) || !ok_vec(x) || !ok_vec(r))
		return FS_ERR_BAD_HANDLE;
	Ctx *ctx = A->ctx;
	if (x->n != A->ncols || r->n != A->nrows || b->n != A->nrows ||
	    x->dtype != r->dtype || b->dtype != r->dtype)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_csr_residual: shapes/dtypes do not match");
	if (x == r)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_csr_residual: x and r must differ");
	if (A->shell_fn) {
		// op::core::residual (operators/core.hh:129-142): apply, then r = b - r
		FS_TRY(shell_apply(A, x, r));
		return fs_vec_subtract(bh, rh, rh);
	}
	if (A->nrows == 0)
		return FS_OK;
	FS_TRY(ensure_sym(A, x->dtype == FS_F32));
	if (x->dtype == FS_F64)
		return launch_spmv<double, false, false>(
			ctx, A, A->val, (const double *)x->d, nullptr,
			EpiResidual<double>{(const double *)b->d, (double *)r->d});
	FS_TRY(ensure_val32(A));
	return launch_spmv<float, false, false>(
		ctx, A, A->val32, (const float *)x->d, nullptr,
		EpiResidual<float>{(const float *)b->d, (float *)r->d});
}

FS_API int fs_csr_diag_inv(fs_csr h, fs_vec dh) {
	Csr *A = reinterpret_cast<Csr *>(h);
	Vec *d = reinterpret_cast<Vec *>(dh);
	if (!ok_csr(A) || !ok_vec(d))
		return FS_ERR_BAD_HANDLE;
	if (d->n != A->nrows)
		return set_err(A->ctx, FS_ERR_SIZE_MISMATCH, "fs_csr_diag_inv: size mismatch");
	FS_TRY(ensure_dinv(A));
	if (A->nrows == 0)
		return FS_OK;
	FS_CUDA_TRY(A->ctx, cudaMemcpyAsync(d->d, d->dtype == FS_F64 ? (void *)A->dinv : (void *)A->dinv32,
	                                    d->bytes(), cudaMemcpyDeviceToDevice, A->ctx->stream));
	return FS_OK;
}

FS_API int fs_parcsr_spmv(fs_csr h, int parts, fs_vec xh, fs_vec yh) {
	Csr *A = reinterpret_cast<Csr *>(h);
	Vec *x = reinterpret_cast<Vec *>(xh), *y = reinterpret_cast<Vec *>(yh);
	if (!ok_csr(A) || !ok_vec(x) || !ok_vec(y))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_parcsr_spmv"));
	Ctx *ctx = A->ctx;
	if (parts < 1 || parts > A->nrows)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_parcsr_spmv: parts must be in [1, nrows]");
	if (x->n != A->ncols || y->n != A->nrows || x->dtype != FS_F64 || y->dtype != FS_F64 ||
	    A->nrows != A->ncols)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_parcsr_spmv: square FP64 operator and vectors required");
	if (x == y)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_parcsr_spmv: x and y must differ");
	parcsr_kernel<true><<<grid_for(ctx, A->nrows, 256, 1), 256, 0, ctx->stream>>>(
		(int)A->nrows, parts, A->rowptr, A->col, A->val, (const double *)x->d, (double *)y->d);
	return check_launch(ctx, "parcsr spmv");
}

FS_API int fs_csr_spmv_transpose(fs_csr h, fs_vec xh, fs_vec yh) {
	Csr *A = reinterpret_cast<Csr *>(h);
	Vec *x = reinterpret_cast<Vec *>(xh), *y = reinterpret_cast<Vec *>(yh);
	if (!ok_csr(A) || !ok_vec(x) || !ok_vec(y))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_csr_spmv_transpose"));
	if (x->n != A->nrows || y->n != A->ncols || x->dtype != FS_F64 || y->dtype != FS_F64)
		return set_err(A->ctx, FS_ERR_SIZE_MISMATCH, "fs_csr_spmv_transpose: FP64 vectors of A^T shape required");
	if (x == y)
		return set_err(A->ctx, FS_ERR_INVALID_ARG, "fs_csr_spmv_transpose: x and y must differ");
	if (A->ncols == 0)
		return FS_OK;
	return transpose_spmv(A, (const double *)x->d, (double *)y->d);
}

}  // extern "C"
