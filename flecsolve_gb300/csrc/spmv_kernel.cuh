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
// Staging: one thread of the CTA copies a row block's contiguous nonzero
// span, its indices and its row offsets into a ring of shared-memory stages
// with bulk asynchronous copies (cp.async.bulk, completed on one mbarrier per
// stage) while the CTA sums an earlier block; one thread per row then
// accumulates its row out of shared memory, with x gathered through the
// read-only path (x of a stencil operator is re-used by neighbouring blocks
// out of L2).  Every wait on an mbarrier is bounded: past the limit the CTA
// records an error in the context's device error word, waits (again bounded)
// for the copies it issued, and finishes without summing further blocks.
//
// This kernel reads 32-bit column ids.  Matrices whose rows follow a few
// column-offset patterns (stencil operators) use the row-pattern kernel of
// spmv_pat.cuh instead; both give the same bits.
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
	unsigned *err;                          // device error word of the context
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

// One pipeline stage: the 16-byte aligned covers of a row block's values,
// column ids and row offsets, plus the block's bounds.  Every array starts on
// a 16-byte boundary.
template<class V>
struct alignas(16) Stage {
	V val[kBlkNnz + 16 / sizeof(V)];
	int col[kBlkNnz + 4];
	int rp[kBlkRows + 1 + 7];
	int r0, r1, k0, k1;
};

// pipeline depth: <= 48 KB of stages per CTA
template<class V>
constexpr int kStages = sizeof(V) == 8 ? 2 : 3;

template<class V>
constexpr size_t spmv_smem_bytes() {
	return sizeof(Stage<V>) * kStages<V>;
}

// ------------------------------------------------- mbarrier / bulk copy --

__device__ __forceinline__ unsigned smem_addr(const void *p) {
	return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count)
	             : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
	asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)),
	             "r"(bytes)
	             : "memory");
}
// bounded wait for the phase with the given parity; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
	const unsigned a = smem_addr(bar);
	for (int it = 0; it < (1 << 22); ++it) {
		unsigned done;
		asm volatile(
			"{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
			" selp.u32 %0, 1, 0, p;\n}\n"
			: "=r"(done)
			: "r"(a), "r"(parity)
			: "memory");
		if (done)
			return true;
	}
	return false;
}
// global -> shared bulk copy of `bytes` (a multiple of 16, both addresses
// 16-byte aligned), completing on `bar`
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         unsigned long long *bar) {
	asm volatile(
		"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
			smem_addr(dst)),
		"l"(src), "r"(bytes), "r"(smem_addr(bar))
		: "memory");
}

// read-only loads that ask L2 to fetch the whole 256-byte group around the
// address (streams whose neighbouring bytes are read by other warps soon)
__device__ __forceinline__ float ld_stream(const float *p) {
	float v;
	asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
	return v;
}
__device__ __forceinline__ double ld_stream(const double *p) {
	double v;
	asm("ld.global.nc.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p));
	return v;
}
__device__ __forceinline__ unsigned char ld_stream(const unsigned char *p) {
	unsigned short v;
	asm("ld.global.nc.L2::256B.u8 %0, [%1];" : "=h"(v) : "l"(p));
	return (unsigned char)v;
}

// 16 bytes (four floats / two doubles) from a 16-byte aligned address,
// through the read-only path
__device__ __forceinline__ void ld_vec16(const float *p, float (&o)[4]) {
	const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
	o[0] = t.x;
	o[1] = t.y;
	o[2] = t.z;
	o[3] = t.w;
}
__device__ __forceinline__ void ld_vec16(const double *p, double (&o)[2]) {
	const double2 t = __ldg(reinterpret_cast<const double2 *>(p));
	o[0] = t.x;
	o[1] = t.y;
}

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// x gather, optionally scaled on the fly by a diagonal (y = A D x, used for
// right Jacobi preconditioning without materialising D x)
template<class V, bool SCALE>
__device__ __forceinline__ V xg(const V *__restrict__ x, const V *__restrict__ d, int c) {
	if constexpr (SCALE)
		return mul_rn(__ldg(d + c), __ldg(x + c));
	else
		return __ldg(x + c);
}

// Issue the bulk copies of a row block (bounds m = {r0, r1, k0, k1}) into
// stage `st`; thread 0 only.  Each cover starts at an aligned index <= the
// first element and ends within 16 bytes past the last, inside the padded
// allocations.  A long row copies nothing (it is summed from global memory).
template<class V>
__device__ __forceinline__ void stage_issue(const CsrDev<V> &A, int4 m, Stage<V> &st,
                                            unsigned long long *bar) {
	constexpr int VW = 16 / sizeof(V);
	const int r0 = m.x, r1 = m.y, k0 = m.z, k1 = m.w;
	st.r0 = r0;
	st.r1 = r1;
	st.k0 = k0;
	st.k1 = k1;
	unsigned bv = 0, bc = 0, br = 0;
	const int a0 = k0 & ~(VW - 1), c0 = k0 & ~3, p0 = r0 & ~3;
	if (k1 - k0 <= kBlkNnz) {
		bv = k1 > k0 ? (unsigned)(((k1 - a0 + VW - 1) / VW) * 16) : 0u;
		bc = k1 > k0 ? (unsigned)(((k1 - c0 + 3) / 4) * 16) : 0u;
		br = (unsigned)(((r1 + 1 - p0 + 3) / 4) * 16);
	}
	mbar_arrive_expect_tx(bar, bv + bc + br);
	if (bv)
		bulk_g2s(st.val, A.val + a0, bv, bar);
	if (bc)
		bulk_g2s(st.col, A.col + c0, bc, bar);
	if (br)
		bulk_g2s(st.rp, A.rowptr + p0, br, bar);
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
// kStages-deep ring: the copies of block i + kStages - 1 are in flight while
// block i is summed out of shared memory.
template<class V, bool EXACT, bool SCALE, class Epi>
__global__ void __launch_bounds__(kBlkRows)
spmv_rb_kernel(CsrDev<V> A, const V *__restrict__ x, const V *__restrict__ dscale, Epi epi) {
	constexpr int NV = Epi::NV;
	constexpr int S = kStages<V>;
	constexpr int VW = 16 / sizeof(V);
	using St = Stage<V>;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	St *stages = reinterpret_cast<St *>(smem_raw);
	__shared__ double red[128];
	__shared__ unsigned long long bars[S];
	__shared__ int abort_flag;
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	Acc<V, NV> acc;
	acc.init();
	const int tid = threadIdx.x;
	const int nb = A.nblk > (int)blockIdx.x ? (A.nblk - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
	if (tid == 0) {
		abort_flag = 0;
#pragma unroll
		for (int s = 0; s < S; ++s)
			mbar_init(&bars[s], 1);
		mbar_init_fence();
	}
	__syncthreads();
	// bounds are loaded one block before their copies are issued, so the
	// issue never waits on a global load
	int4 mnext = make_int4(0, 0, 0, 0);
	if (tid == 0) {
#pragma unroll
		for (int i = 0; i < S - 1; ++i)
			if (i < nb)
				stage_issue<V>(A, block_meta(A, i, nb), stages[i], &bars[i]);
		mnext = block_meta(A, S - 1, nb);
	}
	int i = 0;
	for (; i < nb; ++i) {
		const int ni = i + S - 1;
		if (tid == 0 && ni < nb) {
			stage_issue<V>(A, mnext, stages[ni % S], &bars[ni % S]);
			mnext = block_meta(A, ni + 1, nb);
		}
		if (!mbar_wait(&bars[i % S], (unsigned)((i / S) & 1)))
			abort_flag = 1;
		__syncthreads();
		if (abort_flag)
			break;
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
				const int p0 = r0 & ~3, a0 = k0 & ~(VW - 1);
				const int kb = st.rp[r - p0];
				V s = V(0);
				const int c0 = k0 & ~3;
				const int ke = st.rp[r + 1 - p0];
				// batches of 8: all gathers of a batch are issued before the
				// first product, so a 7-point row costs one L2 round trip
				for (int kc = kb; kc < ke; kc += 8) {
					V a[8], xv[8];
#pragma unroll
					for (int j = 0; j < 8; ++j)
						if (kc + j < ke) {
							a[j] = st.val[kc + j - a0];
							xv[j] = xg<V, SCALE>(x, dscale, st.col[kc + j - c0]);
						}
#pragma unroll
					for (int j = 0; j < 8; ++j)
						if (kc + j < ke) {
							if constexpr (EXACT)
								s = add_rn(s, mul_rn(a[j], xv[j]));
							else
								s = fma(a[j], xv[j], s);
						}
				}
				epi.row(r, s, acc);
			}
		}
		__syncthreads();
	}
	if (i < nb) {
		// a wait ran out: report it, and let the copies this CTA issued land
		// before it exits (bounded as well)
		if (tid == 0) {
			atomicOr(A.err, 1u);
			for (int j = i; j < nb && j < i + S; ++j)
				mbar_wait(&bars[j % S], (unsigned)((j / S) & 1));
		}
		__syncthreads();
	}
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
template<class V, bool EXACT, bool SCALE, class Epi>
static inline int launch_spmv_as(Ctx *ctx, const CsrDev<V> &d, const V *x, const V *dscale,
                                 const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	constexpr size_t smem = spmv_smem_bytes<V>();
	auto kern = spmv_rb_kernel<V, EXACT, SCALE, Epi>;
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
	return check_launch_rc(ctx, launch_pdl(ctx->stream, kern, g, kBlkRows, smem, d, x, dscale, epi),
	                       "spmv");
}

}  // namespace fsg

#include "spmv_pat.cuh"
#include "spmv_sym.cuh"
#include "spmv_grid.cuh"
#include "spmv_fvm.cuh"
#include "spmv_vec.cuh"

namespace fsg {

// The index format in use: the symmetric storage when it is built for the
// current values (and `vals` are A's own values), the general grid storage of
// a grid stencil with asymmetric values, else the warp-specialised row-pattern
// kernel when the matrix carries patterns, else column ids.
template<class V, bool EXACT, bool SCALE, class Epi>
static inline int launch_spmv(Ctx *ctx, const Csr *A, const V *vals, const V *x,
                              const V *dscale, const Epi &epi) {
	constexpr bool F32 = std::is_same_v<V, float>;
	if (A->fvm) {  // matrix-free finite-volume operator
		if constexpr (SCALE)
			return launch_spmv_fvm<V>(ctx, A->fvm, GatherScale<V>{x, dscale}, epi);
		else
			return launch_spmv_fvm<V>(ctx, A->fvm, GatherX<V>{x}, epi);
	}
	const int coding = active_coding(A, F32);
	const bool own_vals = vals == (F32 ? (const V *)A->val32 : (const V *)A->val);
	if (coding == kCodingGrid && own_vals && grid_aligned<V>(A, x, dscale)) {
		if constexpr (SCALE)
			return launch_spmv_grid<V, EXACT, false>(ctx, A, GatherScale<V>{x, dscale}, epi);
		else
			return launch_spmv_grid<V, EXACT, false>(ctx, A, GatherX<V>{x}, epi);
	}
	if (coding == kCodingGridGen && own_vals && grid_aligned<V>(A, x, dscale)) {
		if constexpr (SCALE)
			return launch_spmv_grid<V, EXACT, true>(ctx, A, GatherScale<V>{x, dscale}, epi);
		else
			return launch_spmv_grid<V, EXACT, true>(ctx, A, GatherX<V>{x}, epi);
	}
	if ((coding == kCodingSym || coding == kCodingGrid) && own_vals) {
		if constexpr (SCALE)
			return launch_spmv_sym<V, EXACT>(ctx, A, GatherScale<V>{x, dscale}, epi);
		else
			return launch_spmv_sym<V, EXACT>(ctx, A, GatherX<V>{x}, epi);
	}
	if (coding != kCodingColIds) {
		if constexpr (SCALE)
			return launch_spmv_pat<V, EXACT>(ctx, A, vals, GatherScale<V>{x, dscale}, epi);
		else
			return launch_spmv_pat<V, EXACT>(ctx, A, vals, GatherX<V>{x}, epi);
	}
	if constexpr (!EXACT) {
		const int lanes = spmv_lanes(ctx, A, F32);
		if (lanes > 0)
			return launch_spmv_vec<V, SCALE, Epi>(ctx, A, vals, x, dscale, epi, lanes);
	}
	CsrDev<V> d{A->rowptr, A->col, vals, A->blkinfo, A->nblk, ctx->dev_err};
	return launch_spmv_as<V, EXACT, SCALE, Epi>(ctx, d, x, dscale, epi);
}

}  // namespace fsg
