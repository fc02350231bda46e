// Row-pattern SpMV, warp-specialised.
//
// Same operator and row loop as spmv_rb_kernel (the reference's
// compressed_ops::spmv row loop, flecsolve/matrices/seq.hh:177-193), for
// matrices whose rows follow at most kMaxPat sequences of column offsets
// c - r of at most kPatW nonzeros (stencil operators).  Each row stores the
// 8-bit id of its sequence; a block stores, per warp, where the nonzeros of
// the warp's first row start (the other rows follow from a warp scan of the
// pattern lengths), so neither column ids nor row offsets are read.
//
// A CTA is one producer warp and kPatConsumers consumer warps.  The producer
// (one lane) copies each row block's values, pattern ids and warp offsets into
// a ring of shared-memory stages with bulk asynchronous copies, completing on
// the stage's `full` mbarrier, as soon as the consumers have released the
// stage on its `empty` mbarrier.  Each consumer warp sums 32 rows of the
// block, one row per lane, gathering x through the read-only path (a stencil
// operator re-reads x of neighbouring rows out of L1/L2), and releases the
// stage.  No CTA-wide barrier is taken inside the loop.  Every wait is
// bounded: past the limit the warp records an error in the context's device
// error word and the CTA winds down; the producer waits (bounded) for its
// copies in flight before the CTA exits.
//
// The x value of column c comes from a gather policy: x[c] (y = A x) or
// d[c] x[c] (y = A D x).
//
// Every row sums the same products in the same order as spmv_rb_kernel (FMA,
// or EXACT: rounded products summed left to right), so y is identical bit for
// bit; fused reductions group rows by CTA.
#pragma once

namespace fsg {

constexpr int kPatConsumers = kBlkRows / 32;  // consumer warps, one row per lane
constexpr int kPatThreads = kBlkRows + 32;    // plus the producer warp

template<class V>
struct CsrPat {
	const V *__restrict__ val;
	const int4 *__restrict__ info;           // per block {r0, r1, k0, k1}
	const short *__restrict__ wb;            // per block, per warp: first nonzero - k0
	const unsigned char *__restrict__ pid;   // pattern id per row
	const int *__restrict__ ptab;            // kPatW offsets per pattern
	const unsigned char *__restrict__ plen;  // nonzeros per pattern
	int nblk, npat;
	unsigned *err;
};

template<class V>
struct alignas(16) PatStage {
	V val[kBlkNnz + 16 / sizeof(V)];
	unsigned char pid[kBlkRows + 32];
	short wb[kPatConsumers];
	int4 m;
};

template<class V>
constexpr int kPatStages = sizeof(V) == 4 ? 4 : 3;

template<class V>
constexpr size_t spmv_pat_smem_bytes() {
	return sizeof(PatStage<V>) * kPatStages<V> + sizeof(int) * kMaxPat * kPatW + kMaxPat;
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}

// y = A x
template<class V>
struct GatherX {
	const V *x;
	__device__ void init() {}
	__device__ V at(int c) const { return __ldg(x + c); }
	// the same value, read with a 256-byte L2 fetch (contiguous sweeps)
	__device__ V at_stream(int c) const { return ld_stream(x + c); }
	// 16 bytes from x + c (c a multiple of 16 / sizeof(V), x 16-byte aligned)
	template<int W>
	__device__ void at_vec(int c, V (&o)[W]) const { ld_vec16(x + c, o); }
	__device__ bool aligned16() const { return ((uintptr_t)x & 15) == 0; }
};

// y = A D x (right Jacobi preconditioning without materialising D x); the
// product is rounded once, as in the column-id kernel
template<class V>
struct GatherScale {
	const V *x, *d;
	__device__ void init() {}
	__device__ V at(int c) const { return mul_rn(__ldg(d + c), __ldg(x + c)); }
	__device__ V at_stream(int c) const { return mul_rn(ld_stream(d + c), ld_stream(x + c)); }
	template<int W>
	__device__ void at_vec(int c, V (&o)[W]) const {
		V dv[W];
		ld_vec16(d + c, dv);
		ld_vec16(x + c, o);
#pragma unroll
		for (int q = 0; q < W; ++q)
			o[q] = mul_rn(dv[q], o[q]);
	}
	__device__ bool aligned16() const { return (((uintptr_t)x | (uintptr_t)d) & 15) == 0; }
};

// Issue the copies of row block `b` (bounds m) into stage `st`; the
// producer's lane only.  Values and pattern ids use the 16-byte aligned
// covers of the padded arrays.
template<class V>
__device__ __forceinline__ void pat_issue(const CsrPat<V> &A, int b, int4 m, PatStage<V> &st,
                                          unsigned long long *bar) {
	constexpr int VW = 16 / sizeof(V);
	const int r0 = m.x, r1 = m.y, k0 = m.z, k1 = m.w;
	st.m = m;  // published by the arrive below (release), read after the wait
	const int a0 = k0 & ~(VW - 1), q0 = r0 & ~15;
	const unsigned bv = k1 > k0 ? (unsigned)(((k1 - a0 + VW - 1) / VW) * 16) : 0u;
	const unsigned bp = (unsigned)(((r1 - q0 + 15) / 16) * 16);
	mbar_arrive_expect_tx(bar, bv + bp + (unsigned)sizeof(st.wb));
	if (bv)
		bulk_g2s(st.val, A.val + a0, bv, bar);
	bulk_g2s(st.pid, A.pid + q0, bp, bar);
	bulk_g2s(st.wb, A.wb + (size_t)b * kPatConsumers, (unsigned)sizeof(st.wb), bar);
}

template<class V, bool EXACT, class G, class Epi, int S>
__global__ void __launch_bounds__(kPatThreads)
spmv_pat_kernel(CsrPat<V> A, G g_in, Epi epi) {
	constexpr int NV = Epi::NV;
	constexpr int VW = 16 / sizeof(V);
	using St = PatStage<V>;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	St *stages = reinterpret_cast<St *>(smem_raw);
	int *ptab = reinterpret_cast<int *>(smem_raw + sizeof(St) * S);
	unsigned char *plen = reinterpret_cast<unsigned char *>(ptab + kMaxPat * kPatW);
	__shared__ double red[128];
	__shared__ unsigned long long full[S], empty[S];
	__shared__ int abort_flag;
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	G g = g_in;
	g.init();
	Acc<V, NV> acc;
	acc.init();
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int nb = A.nblk > (int)blockIdx.x ? (A.nblk - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
	if (tid == 0) {
		abort_flag = 0;
#pragma unroll
		for (int s = 0; s < S; ++s) {
			mbar_init(&full[s], 1);
			mbar_init(&empty[s], kPatConsumers);
		}
		mbar_init_fence();
	}
	for (int i = tid; i < A.npat * kPatW; i += blockDim.x)
		ptab[i] = __ldg(A.ptab + i);
	for (int i = tid; i < A.npat; i += blockDim.x)
		plen[i] = __ldg(A.plen + i);
	__syncthreads();
	volatile int *abort_v = &abort_flag;
	if (warp == kPatConsumers) {
		// producer
		if (lane == 0) {
			int issued = 0;
			int4 m = nb > 0 ? __ldg(A.info + blockIdx.x) : make_int4(0, 0, 0, 0);
			for (int i = 0; i < nb; ++i) {
				const int s = i % S;
				if (i >= S && !mbar_wait(&empty[s], (unsigned)(((i / S) - 1) & 1))) {
					atomicOr(A.err, 1u);
					*abort_v = 1;
					break;
				}
				if (*abort_v)
					break;
				const int b = (int)blockIdx.x + i * (int)gridDim.x;
				const int4 mn = i + 1 < nb ? __ldg(A.info + b + gridDim.x) : make_int4(0, 0, 0, 0);
				pat_issue<V>(A, b, m, stages[s], &full[s]);
				issued = i + 1;
				m = mn;
			}
			// every copy lands before the CTA exits (completed phases return
			// at once)
			for (int j = issued > S ? issued - S : 0; j < issued; ++j)
				mbar_wait(&full[j % S], (unsigned)((j / S) & 1));
		}
	}
	else {
		for (int i = 0; i < nb; ++i) {
			const int s = i % S;
			// every lane waits; the outcome is made warp-uniform so no lane
			// leaves the warp's shuffles below
			if (!__all_sync(0xffffffffu, mbar_wait(&full[s], (unsigned)((i / S) & 1)))) {
				if (lane == 0) {
					atomicOr(A.err, 1u);
					*abort_v = 1;
				}
				break;
			}
			const St &st = stages[s];
			const int4 m = st.m;
			const int r0 = m.x, r1 = m.y, k0 = m.z;
			const int r = r0 + warp * 32 + lane;
			int len = 0, pp = 0;
			if (r < r1) {
				pp = st.pid[r - (r0 & ~15)];
				len = plen[pp];
			}
			int incl = len;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const int t = __shfl_up_sync(0xffffffffu, incl, o);
				if (lane >= o)
					incl += t;
			}
			if (r < r1) {
				const V *vv = st.val + (k0 - (k0 & ~(VW - 1))) + st.wb[warp] + (incl - len);
				const int4 o0 = *reinterpret_cast<const int4 *>(ptab + pp * kPatW);
				const int4 o1 = *reinterpret_cast<const int4 *>(ptab + pp * kPatW + 4);
				const int off[kPatW] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z, o1.w};
				V a[kPatW], xv[kPatW];
#pragma unroll
				for (int j = 0; j < kPatW; ++j)
					if (j < len) {
						a[j] = vv[j];
						xv[j] = g.at(r + off[j]);
					}
				V sum = V(0);
#pragma unroll
				for (int j = 0; j < kPatW; ++j)
					if (j < len) {
						if constexpr (EXACT)
							sum = add_rn(sum, mul_rn(a[j], xv[j]));
						else
							sum = fma(a[j], xv[j], sum);
					}
				epi.row(r, sum, acc);
			}
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&empty[s]);
			if (__any_sync(0xffffffffu, *abort_v != 0))
				break;
		}
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

template<class V, bool EXACT, class G, class Epi>
static inline int launch_spmv_pat(Ctx *ctx, const Csr *A, const V *vals, const G &g,
                                  const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	constexpr int S = kPatStages<V>;
	constexpr size_t smem = spmv_pat_smem_bytes<V>();
	auto kern = spmv_pat_kernel<V, EXACT, G, Epi, S>;
	if (per_sm == 0) {
		if (smem > 48 * 1024 &&
		    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
		        cudaSuccess)
			return set_err(ctx, FS_ERR_CUDA, "spmv: cannot reserve %zu bytes of shared memory", smem);
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kPatThreads, smem) != cudaSuccess ||
		    nb < 1)
			nb = 1;
		per_sm = nb;
	}
	CsrPat<V> d{vals, A->blkinfo, A->pwb, A->pid, A->ptab, A->plen, A->nblk, A->npat, ctx->dev_err};
	const int grid = spmv_grid(ctx, A->nblk, per_sm);
	return check_launch_rc(ctx, launch_pdl(ctx->stream, kern, grid, kPatThreads, smem, d, g, epi),
	                       "spmv (row patterns)");
}

}  // namespace fsg
