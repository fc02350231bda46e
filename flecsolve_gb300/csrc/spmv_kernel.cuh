// Row-block ("CSR-stream") SpMV kernel template with fused epilogues.
//
// Replaces the serial row loop of mat::compressed_ops::spmv
// (flecsolve/matrices/seq.hh:177-193).  The matrix rows are cut once, at
// creation, into blocks of at most kBlkRows rows and kBlkNnz nonzeros (row-
// length binning: a row longer than kBlkNnz forms a block of its own and is
// summed by the whole CTA).  A persistent grid walks the blocks with a static
// stride, so every partial sum has a fixed owner and the reductions fused into
// the epilogue are deterministic.
//
// Per block: the contiguous nonzero span [rowptr[r0], rowptr[r1]) is staged
// into shared memory with coalesced loads (the values with 16-byte vector
// loads), then one thread per row accumulates its row from shared memory with
// x gathered through the read-only path (x of a 7-point stencil is re-used by
// neighbouring blocks out of L2).
//
// EXACT mode stages the rounded products a_k * x[c_k] instead and sums them
// left to right per row, which is the reference's operation order bit for bit.
#pragma once

#include <type_traits>

#include "fsgpu_internal.cuh"

namespace fsg {

template<class V>
struct CsrDev {
	const int *__restrict__ rowptr;
	const int *__restrict__ col;
	const V *__restrict__ val;
	const int *__restrict__ blk;
	int nblk;
};

// Per-thread accumulators for fused reductions: plain FP64 fma for double
// vectors, compensated two-sum/two-product pairs for float vectors.
template<int NV>
struct AccD {
	double v[NV > 0 ? NV : 1];
	__device__ __forceinline__ void init() {
#pragma unroll
		for (int k = 0; k < (NV > 0 ? NV : 1); ++k)
			v[k] = 0.0;
	}
	__device__ __forceinline__ void add_prod(int k, double a, double b) {
		v[k] = fma(a, b, v[k]);
	}
	// block tree -> part[blockIdx.x * NV + k]
	__device__ __forceinline__ void to_part(double *part, double *sh) {
		if constexpr (NV > 0) {
			block_sum<NV>(v, sh);
			if (threadIdx.x == 0)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					part[(size_t)blockIdx.x * NV + k] = v[k];
		}
	}
};

template<int NV>
struct AccF {
	cf32 v[NV > 0 ? NV : 1];
	__device__ __forceinline__ void init() {
#pragma unroll
		for (int k = 0; k < (NV > 0 ? NV : 1); ++k)
			v[k] = cf32{0.f, 0.f};
	}
	__device__ __forceinline__ void add_prod(int k, float a, float b) {
		v[k].add_prod(a, b);
	}
	__device__ __forceinline__ void to_part(double *part, double *sh) {
		if constexpr (NV > 0) {
			block_sum_cf<NV>(v, reinterpret_cast<float *>(sh));
			if (threadIdx.x == 0)
#pragma unroll
				for (int k = 0; k < NV; ++k)
					part[(size_t)blockIdx.x * NV + k] =
						(double)v[k].hi + (double)v[k].lo;
		}
	}
};

template<class V, int NV>
using Acc = std::conditional_t<std::is_same_v<V, double>, AccD<NV>, AccF<NV>>;

// shared staging: values (or products) and column ids of one row block
template<class V>
struct SpmvSmem {
	V val[kBlkNnz];
	int col[kBlkNnz];
	double red[128];
};

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

// x gather, optionally scaled on the fly by a diagonal (y = A D x, used for
// right Jacobi preconditioning without materialising D x)
template<class V, bool SCALE>
__device__ __forceinline__ V xg(const V *__restrict__ x, const V *__restrict__ d, int c) {
	if constexpr (SCALE)
		return mul_rn(__ldg(d + c), __ldg(x + c));
	else
		return __ldg(x + c);
}

// Epilogue concept (struct with):
//   static constexpr int NV;                        fused reductions
//   __device__ bool skip() const;                   uniform early exit
//   __device__ void row(int r, V s, Acc<V,NV>& acc) consume row result
//   __device__ void finish(const double* sums)      last block, thread 0
//   double* part; unsigned* counter;                reduction scratch
template<class V, bool EXACT, bool SCALE, class Epi>
__global__ void __launch_bounds__(kBlkRows)
spmv_rb_kernel(CsrDev<V> A, const V *__restrict__ x, const V *__restrict__ dscale,
               Epi epi) {
	constexpr int NV = Epi::NV;
	__shared__ SpmvSmem<V> sm;
	if (epi.skip())
		return;
	Acc<V, NV> acc;
	acc.init();
	const int tid = threadIdx.x;
	for (int b = blockIdx.x; b < A.nblk; b += gridDim.x) {
		const int r0 = A.blk[b], r1 = A.blk[b + 1];
		const int k0 = A.rowptr[r0], k1 = A.rowptr[r1];
		const int span = k1 - k0;
		if (span > kBlkNnz) {
			// a single long row: the CTA sums it (fixed strided order + tree)
			V s = V(0);
			if constexpr (EXACT) {
				// chunks of products summed left to right by thread 0
				for (int c0 = k0; c0 < k1; c0 += kBlkNnz) {
					int c1 = min(k1, c0 + kBlkNnz);
					for (int k = c0 + tid; k < c1; k += blockDim.x)
						sm.val[k - c0] = mul_rn(A.val[k], xg<V, SCALE>(x, dscale, A.col[k]));
					__syncthreads();
					if (tid == 0)
						for (int k = 0; k < c1 - c0; ++k)
							s = add_rn(s, sm.val[k]);
					__syncthreads();
				}
			}
			else {
				double t[1] = {0.0};
				for (int k = k0 + tid; k < k1; k += blockDim.x)
					t[0] = fma((double)A.val[k], (double)xg<V, SCALE>(x, dscale, A.col[k]), t[0]);
				block_sum<1>(t, sm.red);
				s = (V)t[0];
				__syncthreads();
			}
			if (tid == 0)
				epi.row(r0, s, acc);
			continue;
		}
		// stage the block's nonzeros
		if constexpr (EXACT) {
			for (int k = k0 + tid; k < k1; k += blockDim.x)
				sm.val[k - k0] = mul_rn(A.val[k], xg<V, SCALE>(x, dscale, A.col[k]));
		}
		else {
			// 16-byte vector loads over the aligned cover of [k0, k1)
			constexpr int VW = 16 / sizeof(V);
			using VT = std::conditional_t<std::is_same_v<V, double>, double2, float4>;
			const int a0 = k0 & ~(VW - 1);
			for (int k = a0 + tid * VW; k < k1; k += blockDim.x * VW) {
				VT q = __ldg(reinterpret_cast<const VT *>(A.val + k));
				const V *qv = reinterpret_cast<const V *>(&q);
#pragma unroll
				for (int e = 0; e < VW; ++e)
					if (k + e >= k0 && k + e < k1)
						sm.val[k + e - k0] = qv[e];
			}
			const int c0 = k0 & ~3;
			for (int k = c0 + tid * 4; k < k1; k += blockDim.x * 4) {
				int4 q = __ldg(reinterpret_cast<const int4 *>(A.col + k));
				const int *qc = reinterpret_cast<const int *>(&q);
#pragma unroll
				for (int e = 0; e < 4; ++e)
					if (k + e >= k0 && k + e < k1)
						sm.col[k + e - k0] = qc[e];
			}
		}
		__syncthreads();
		const int r = r0 + tid;
		if (r < r1) {
			const int a = A.rowptr[r] - k0, e = A.rowptr[r + 1] - k0;
			V s = V(0);
			if constexpr (EXACT) {
				for (int k = a; k < e; ++k)
					s = add_rn(s, sm.val[k]);
			}
			else {
				for (int k = a; k < e; ++k)
					s = fma(sm.val[k], xg<V, SCALE>(x, dscale, sm.col[k]), s);
			}
			epi.row(r, s, acc);
		}
		__syncthreads();
	}
	if constexpr (NV > 0) {
		acc.to_part(epi.part, sm.red);
		if (last_block(epi.counter)) {
			double sums[NV];
			sum_partials<NV>(epi.part, gridDim.x, sums, sm.red);
			if (tid == 0) {
				epi.finish(sums);
				*epi.counter = 0;
			}
		}
	}
}

// plain y = A x
template<class V>
struct EpiStore {
	static constexpr int NV = 0;
	V *y;
	double *part = nullptr;
	unsigned *counter = nullptr;
	__device__ bool skip() const { return false; }
	template<class A>
	__device__ void row(int r, V s, A &) const { y[r] = s; }
	__device__ void finish(const double *) const {}
};

// r = b - A x
template<class V>
struct EpiResidual {
	static constexpr int NV = 0;
	const V *b;
	V *y;
	double *part = nullptr;
	unsigned *counter = nullptr;
	__device__ bool skip() const { return false; }
	template<class A>
	__device__ void row(int r, V s, A &) const { y[r] = b[r] - s; }
	__device__ void finish(const double *) const {}
};

// grid size of the persistent SpMV for this matrix
int spmv_grid(Ctx *ctx, int nblk);

template<class V, bool EXACT, bool SCALE, class Epi>
inline int launch_spmv(Ctx *ctx, const Csr *A, const V *vals, const V *x,
                       const V *dscale, const Epi &epi) {
	CsrDev<V> d{A->rowptr, A->col, vals, A->blk, A->nblk};
	int g = spmv_grid(ctx, A->nblk);
	spmv_rb_kernel<V, EXACT, SCALE, Epi><<<g, kBlkRows, 0, ctx->stream>>>(d, x, dscale, epi);
	return check_launch(ctx, "spmv");
}

}  // namespace fsg
