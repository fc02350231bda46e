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
// Per block: the contiguous nonzero span [rowptr[r0], rowptr[r1]) and the
// block's row offsets are copied into shared memory with 16-byte cp.async
// copies of their aligned covers, then one thread per row accumulates its row
// from shared memory with x gathered through the read-only path (x of a
// 7-point stencil is re-used by neighbouring blocks out of L2).
//
// Column-offset coding: when every row block's nonzeros use at most kOffTab
// distinct column offsets c - r (a stencil pattern: 7 for a 7-point
// operator), the matrix also carries a per-block table of those offsets and a
// 4-bit code per nonzero (two per byte), and the kernel reads the codes
// instead of the 32-bit column ids: index traffic 0.5 instead of 4 bytes per
// nonzero.  The columns, the products and their order are the same, so the
// result is the same bit for bit.
//
// EXACT mode rounds every product a_k * x[c_k] and adds the products left to
// right per row, which is the reference's operation order bit for bit.
#pragma once

#include <type_traits>

#include "fsgpu_internal.cuh"

namespace fsg {

template<class V>
struct CsrDev {
	const int *__restrict__ rowptr;
	const int *__restrict__ col;
	const V *__restrict__ val;
	const int4 *__restrict__ info;  // per row block {r0, r1, k0, k1}
	int nblk;
	const unsigned char *__restrict__ code;  // coded: 4-bit offset code per nonzero
	const int *__restrict__ tab;             // coded: kOffTab offsets per row block
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

// One pipeline stage: the 16-byte aligned cover of a row block's values,
// column ids (or offset codes and the block's offset table) and row offsets,
// plus the block's bounds.
template<class V, bool CODED>
struct alignas(16) Stage {
	V val[kBlkNnz + 16 / sizeof(V)];
	int col[CODED ? 4 : kBlkNnz + 4];
	unsigned char code[CODED ? kBlkNnz / 2 + 32 : 16];
	int tab[kOffTab];
	int rp[kBlkRows + 1 + 4];
	int r0, r1, k0, k1;
};

// pipeline depth: plain FP64 2 and FP32 3 (<= 48 KB per CTA); the smaller
// coded stages allow one more
template<class V, bool CODED>
constexpr int kStages = (sizeof(V) == 8 ? 2 : 3) + (CODED ? 1 : 0);

template<class V, bool CODED>
constexpr size_t spmv_smem_bytes() {
	return sizeof(Stage<V, CODED>) * kStages<V, CODED>;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
	const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
	asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template<int N>
__device__ __forceinline__ void cp_async_wait() {
	asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

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

// Issue the asynchronous copies of row block `b` (bounds m = {r0, r1, k0,
// k1}) into stage `st`; every thread commits one group, possibly empty.  All
// global reads stay inside the padded allocations: covers start at an aligned
// index <= the first element and end < last element + 4 (codes: + 16 bytes).
template<class V, bool CODED>
__device__ __forceinline__ void stage_issue(const CsrDev<V> &A, int b, int4 m, Stage<V, CODED> &st,
                                            bool valid) {
	if (valid) {
		constexpr int VW = 16 / sizeof(V);
		const int r0 = m.x, r1 = m.y, k0 = m.z, k1 = m.w;
		if (threadIdx.x == 0) {
			st.r0 = r0;
			st.r1 = r1;
			st.k0 = k0;
			st.k1 = k1;
		}
		if (k1 - k0 <= kBlkNnz) {
			const int a0 = k0 & ~(VW - 1);
			const int nv = (k1 - a0 + VW - 1) / VW;
			for (int c = threadIdx.x; c < nv; c += blockDim.x)
				cp_async16(st.val + c * VW, A.val + a0 + c * VW);
			if constexpr (CODED) {
				const int ab = (k0 >> 1) & ~15;
				const int nb16 = (((k1 + 1) >> 1) - ab + 15) / 16;
				for (int c = threadIdx.x; c < nb16; c += blockDim.x)
					cp_async16(st.code + c * 16, A.code + ab + c * 16);
				if (threadIdx.x < kOffTab / 4)
					cp_async16(st.tab + threadIdx.x * 4, A.tab + (size_t)b * kOffTab + threadIdx.x * 4);
			}
			else {
				const int c0 = k0 & ~3;
				const int nc = (k1 - c0 + 3) / 4;
				for (int c = threadIdx.x; c < nc; c += blockDim.x)
					cp_async16(st.col + c * 4, A.col + c0 + c * 4);
			}
			const int p0 = r0 & ~3;
			const int np = (r1 + 1 - p0 + 3) / 4;
			for (int c = threadIdx.x; c < np; c += blockDim.x)
				cp_async16(st.rp + c * 4, A.rowptr + p0 + c * 4);
		}
	}
	cp_async_commit();
}

// bounds of the i-th row block of this CTA (a dummy past the end)
template<class V>
__device__ __forceinline__ int4 block_meta(const CsrDev<V> &A, int i, int nb) {
	return i < nb ? __ldg(A.info + blockIdx.x + i * gridDim.x) : make_int4(0, 0, 0, 0);
}

// Epilogue concept (struct with):
//   static constexpr int NV;                        fused reductions
//   __device__ bool skip() const;                   uniform early exit
//   __device__ void row(int r, V s, Acc<V,NV>& acc) consume row result
//   __device__ void finish(const double* sums)      last block, thread 0
//   double* part; unsigned* counter;                reduction scratch
//
// Persistent CTAs walk the row blocks b = blockIdx.x + i * gridDim.x through a
// kStages-deep cp.async pipeline: the copies of block i + kStages - 1 are in
// flight while block i is summed out of shared memory.
template<class V, bool EXACT, bool SCALE, class Epi, bool CODED = false>
__global__ void __launch_bounds__(kBlkRows)
spmv_rb_kernel(CsrDev<V> A, const V *__restrict__ x, const V *__restrict__ dscale, Epi epi) {
	constexpr int NV = Epi::NV;
	constexpr int S = kStages<V, CODED>;
	constexpr int VW = 16 / sizeof(V);
	extern __shared__ __align__(16) unsigned char smem_raw[];
	using St = Stage<V, CODED>;
	St *stages = reinterpret_cast<St *>(smem_raw);
	__shared__ double red[128];
	if (epi.skip())
		return;
	Acc<V, NV> acc;
	acc.init();
	const int tid = threadIdx.x;
	const int nb = A.nblk > (int)blockIdx.x ? (A.nblk - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
#pragma unroll
	for (int i = 0; i < S - 1; ++i)
		stage_issue<V, CODED>(A, blockIdx.x + i * gridDim.x, block_meta(A, i, nb), stages[i], i < nb);
	// bounds are loaded one iteration before their copies are issued, so the
	// issue never waits on a global load
	int4 mnext = block_meta(A, S - 1, nb);
	for (int i = 0; i < nb; ++i) {
		const int ni = i + S - 1;
		stage_issue<V, CODED>(A, blockIdx.x + ni * gridDim.x, mnext, stages[ni % S], ni < nb);
		mnext = block_meta(A, ni + 1, nb);
		cp_async_wait<S - 1>();
		__syncthreads();
		const St &st = stages[i % S];
		const int r0 = st.r0, r1 = st.r1, k0 = st.k0, k1 = st.k1;
		if (k1 - k0 > kBlkNnz) {
			// a single long row: the CTA sums it from global memory
			V s = V(0);
			if constexpr (EXACT) {
				if (tid == 0)
					for (int k = k0; k < k1; ++k)
						s = add_rn(s, mul_rn(A.val[k], xg<V, SCALE>(x, dscale, A.col[k])));
			}
			else {
				double t[1] = {0.0};
				for (int k = k0 + tid; k < k1; k += blockDim.x)
					t[0] = fma((double)A.val[k], (double)xg<V, SCALE>(x, dscale, A.col[k]), t[0]);
				block_sum<1>(t, red);
				s = (V)t[0];
			}
			if (tid == 0)
				epi.row(r0, s, acc);
		}
		else {
			const int r = r0 + tid;
			if (r < r1) {
				const int p0 = r0 & ~3, a0 = k0 & ~(VW - 1), c0 = k0 & ~3;
				const int ab = (k0 >> 1) & ~15;
				const int kb = st.rp[r - p0], ke = st.rp[r + 1 - p0];
				V s = V(0);
				// batches of 8: all gathers of a batch are issued before the
				// first product, so a 7-point row costs one L2 round trip
				for (int kc = kb; kc < ke; kc += 8) {
					V a[8], xv[8];
#pragma unroll
					for (int j = 0; j < 8; ++j) {
						if (kc + j < ke) {
							const int k = kc + j;
							a[j] = st.val[k - a0];
							int c;
							if constexpr (CODED) {
								const unsigned byte = st.code[(k >> 1) - ab];
								c = r + st.tab[(k & 1) ? (byte >> 4) : (byte & 15u)];
							}
							else
								c = st.col[k - c0];
							xv[j] = xg<V, SCALE>(x, dscale, c);
						}
					}
#pragma unroll
					for (int j = 0; j < 8; ++j) {
						if (kc + j < ke) {
							if constexpr (EXACT)
								s = add_rn(s, mul_rn(a[j], xv[j]));
							else
								s = fma(a[j], xv[j], s);
						}
					}
				}
				epi.row(r, s, acc);
			}
		}
		__syncthreads();
	}
	cp_async_wait<0>();
	if constexpr (NV > 0) {
		acc.to_part(epi.part, red);
		if (last_block(epi.counter)) {
			double sums[NV];
			sum_partials<NV>(epi.part, gridDim.x, sums, red);
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

// persistent grid: resident CTAs per SM (from the occupancy of this
// instantiation) x SMs, capped by the number of row blocks
int spmv_grid(Ctx *ctx, int nblk, int per_sm);

// `static`: every translation unit has its own copy of the kernel (no
// relocatable device code), so the attribute and the occupancy are set up
// per unit, in a per-unit cache
template<class V, bool EXACT, bool SCALE, class Epi, bool CODED>
static inline int launch_spmv_as(Ctx *ctx, const CsrDev<V> &d, const V *x, const V *dscale,
                                 const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	constexpr size_t smem = spmv_smem_bytes<V, CODED>();
	auto kern = spmv_rb_kernel<V, EXACT, SCALE, Epi, CODED>;
	if (per_sm == 0) {
		if (smem > 48 * 1024 &&
		    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
		        cudaSuccess)
			return set_err(ctx, FS_ERR_CUDA, "spmv: cannot reserve %zu bytes of shared memory", smem);
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kBlkRows, smem) != cudaSuccess ||
		    nb < 1)
			nb = 1;
		per_sm = nb;
	}
	int g = spmv_grid(ctx, d.nblk, per_sm);
	kern<<<g, kBlkRows, smem, ctx->stream>>>(d, x, dscale, epi);
	return check_launch(ctx, "spmv");
}

// the offset-coded kernel when the matrix carries codes, else the plain one
template<class V, bool EXACT, bool SCALE, class Epi>
static inline int launch_spmv(Ctx *ctx, const Csr *A, const V *vals, const V *x,
                       const V *dscale, const Epi &epi) {
	CsrDev<V> d{A->rowptr, A->col, vals, A->blkinfo, A->nblk, A->code, A->tab};
	if (A->code && A->use_codes)
		return launch_spmv_as<V, EXACT, SCALE, Epi, true>(ctx, d, x, dscale, epi);
	return launch_spmv_as<V, EXACT, SCALE, Epi, false>(ctx, d, x, dscale, epi);
}

}  // namespace fsg
