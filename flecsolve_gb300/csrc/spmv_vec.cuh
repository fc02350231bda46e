// Vector SpMV over column ids, for matrices whose rows hold dozens to
// thousands of nonzeros.
//
// Same operator as spmv_rb_kernel (the reference's compressed_ops::spmv row
// loop, flecsolve/matrices/seq.hh:177-193), FMA mode: L lanes share a row
// (L = 4, 8, 16 or 32, chosen per matrix and precision by the autotuner of
// spmv.cu, or from the mean row length while a graph is being captured).
// The lanes stride over the row's nonzeros -- value and column loads
// coalesced across the group and marked streaming (read once: evicted first,
// so that x, gathered at random columns, keeps its place in L2), four
// nonzeros per lane in flight, the x gathers independent of each other --
// and a fixed xor tree over the group adds the lanes' sums.  A warp takes 32 / L consecutive rows per step and
// the warps stride over the rows in a fixed order, so every row has one owner
// and the fused reductions of the epilogue are deterministic.
//
// A fixed L serves rows of one length well; the binned schedule below serves
// rows of many lengths.  The row-block kernel sums each row in one thread
// (the reference's order, the only form of EXACT mode); with long rows its
// blocks hold few rows, so most of its threads idle while one thread walks a
// row gather by gather.
#pragma once

namespace fsg {

constexpr int kVecThreads = 256;

template<class V, int L, bool SCALE, class Epi>
__global__ void __launch_bounds__(kVecThreads)
spmv_vec_kernel(const int *__restrict__ rowptr, const int *__restrict__ col,
                const V *__restrict__ val, int n, const V *__restrict__ x,
                const V *__restrict__ dscale, Epi epi) {
	static_assert(L == 4 || L == 8 || L == 16 || L == 32, "lanes per row");
	constexpr int NV = Epi::NV;
	constexpr int RPW = 32 / L;  // rows per warp and step
	__shared__ double red[128];
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	Acc<V, NV> acc;
	acc.init();
	const int lane = threadIdx.x & 31;
	const int sub = lane & (L - 1);
	const int grp = lane / L;
	const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
	const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
	for (int base = warp * RPW; base < n; base += nwarps * RPW) {
		const int r = base + grp;
		V s = V(0);
		if (r < n) {
			const int k0 = __ldg(rowptr + r), k1 = __ldg(rowptr + r + 1);
			int k = k0 + sub;
			for (; k + 3 * L < k1; k += 4 * L) {
				V a[4], xv[4];
				int c[4];
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					a[j] = __ldcs(val + k + j * L);
					c[j] = __ldcs(col + k + j * L);
				}
#pragma unroll
				for (int j = 0; j < 4; ++j)
					xv[j] = xg<V, SCALE>(x, dscale, c[j]);
#pragma unroll
				for (int j = 0; j < 4; ++j)
					s = fma(a[j], xv[j], s);
			}
			for (; k < k1; k += L)
				s = fma(__ldcs(val + k), xg<V, SCALE>(x, dscale, __ldcs(col + k)), s);
		}
		// every lane of the warp reaches the tree (rows past n add zeros)
#pragma unroll
		for (int o = L / 2; o > 0; o >>= 1)
			s += __shfl_xor_sync(0xffffffffu, s, o);
		if (sub == 0 && r < n)
			epi.row(r, s, acc);
	}
	if constexpr (NV > 0) {
		acc.to_part(epi.part, red);
		if (last_block(epi.counter)) {
			double sums[NV];
			sum_partials<NV>(epi.part, gridDim.x, sums, red);
			if (threadIdx.x == 0) {
				epi.finish(sums);
				*epi.counter = 0;
			}
		}
	}
}

// Binned schedule: the rows grouped by length class (at most 8, 32, 128
// nonzeros, longer) into warp tasks of 32 / L rows of one class, L = 4, 8,
// 16, 32 lanes per row (a long row has a whole warp, short ones share it), so
// the rows of a warp finish together; tasks are taken in a fixed order.
// rows: row ids by class; task: {first slot in rows, L | (rows << 8)}.
template<class V, bool SCALE, class Epi>
__global__ void __launch_bounds__(kVecThreads)
spmv_bin_kernel(const int *__restrict__ rowptr, const int *__restrict__ col,
                const V *__restrict__ val, const int *__restrict__ rows,
                const int2 *__restrict__ task, int ntask, const V *__restrict__ x,
                const V *__restrict__ dscale, Epi epi) {
	constexpr int NV = Epi::NV;
	__shared__ double red[128];
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	Acc<V, NV> acc;
	acc.init();
	const int lane = threadIdx.x & 31;
	const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
	const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
	for (int t = warp; t < ntask; t += nwarps) {
		const int2 d = __ldg(task + t);
		const int L = d.y & 0xff, cnt = d.y >> 8;  // the same for the whole warp
		const int grp = lane / L, sub = lane & (L - 1);
		int r = -1;
		V s = V(0);
		if (grp < cnt) {
			r = __ldg(rows + d.x + grp);
			const int k0 = __ldg(rowptr + r), k1 = __ldg(rowptr + r + 1);
			int k = k0 + sub;
			for (; k + 3 * L < k1; k += 4 * L) {
				V a[4], xv[4];
				int c[4];
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					a[j] = __ldcs(val + k + j * L);
					c[j] = __ldcs(col + k + j * L);
				}
#pragma unroll
				for (int j = 0; j < 4; ++j)
					xv[j] = xg<V, SCALE>(x, dscale, c[j]);
#pragma unroll
				for (int j = 0; j < 4; ++j)
					s = fma(a[j], xv[j], s);
			}
			for (; k < k1; k += L)
				s = fma(__ldcs(val + k), xg<V, SCALE>(x, dscale, __ldcs(col + k)), s);
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1)
			if (o < L)
				s += __shfl_xor_sync(0xffffffffu, s, o);
		if (sub == 0 && r >= 0)
			epi.row(r, s, acc);
	}
	if constexpr (NV > 0) {
		acc.to_part(epi.part, red);
		if (last_block(epi.counter)) {
			double sums[NV];
			sum_partials<NV>(epi.part, gridDim.x, sums, red);
			if (threadIdx.x == 0) {
				epi.finish(sums);
				*epi.counter = 0;
			}
		}
	}
}

template<class V, bool SCALE, class Epi>
static inline int launch_spmv_bin(Ctx *ctx, const Csr *A, const V *vals, const V *x,
                                  const V *dscale, const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	auto kern = spmv_bin_kernel<V, SCALE, Epi>;
	if (per_sm == 0) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kVecThreads, 0) != cudaSuccess ||
		    nb < 1)
			nb = 1;
		per_sm = nb;
	}
	constexpr int warps_per_cta = kVecThreads / 32;
	const int need = (A->bin_ntask + warps_per_cta - 1) / warps_per_cta;
	const int grid = std::max(1, std::min(need, ctx->sms * std::min(per_sm, 8)));
	return check_launch_rc(ctx, launch_pdl(ctx->stream, kern, grid, kVecThreads, 0, A->rowptr,
	                                       A->col, vals, (const int *)A->bin_rows,
	                                       (const int2 *)A->bin_task, A->bin_ntask, x, dscale, epi),
	                       "spmv (vector, rows binned by length)");
}

template<class V, int L, bool SCALE, class Epi>
static inline int launch_spmv_vec_l(Ctx *ctx, const Csr *A, const V *vals, const V *x,
                                    const V *dscale, const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	auto kern = spmv_vec_kernel<V, L, SCALE, Epi>;
	if (per_sm == 0) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kVecThreads, 0) != cudaSuccess ||
		    nb < 1)
			nb = 1;
		per_sm = nb;
	}
	constexpr int rows_per_cta = kVecThreads / L;
	const int need = (int)((A->nrows + rows_per_cta - 1) / rows_per_cta);
	const int grid = std::max(1, std::min(need, ctx->sms * std::min(per_sm, 8)));
	return check_launch_rc(ctx, launch_pdl(ctx->stream, kern, grid, kVecThreads, 0, A->rowptr,
	                                       A->col, vals, (int)A->nrows, x, dscale, epi),
	                       "spmv (vector, column ids)");
}

template<class V, bool SCALE, class Epi>
static inline int launch_spmv_vec(Ctx *ctx, const Csr *A, const V *vals, const V *x,
                                  const V *dscale, const Epi &epi, int lanes) {
	switch (lanes) {
	case 1: return launch_spmv_bin<V, SCALE, Epi>(ctx, A, vals, x, dscale, epi);
	case 4: return launch_spmv_vec_l<V, 4, SCALE, Epi>(ctx, A, vals, x, dscale, epi);
	case 8: return launch_spmv_vec_l<V, 8, SCALE, Epi>(ctx, A, vals, x, dscale, epi);
	case 16: return launch_spmv_vec_l<V, 16, SCALE, Epi>(ctx, A, vals, x, dscale, epi);
	default: return launch_spmv_vec_l<V, 32, SCALE, Epi>(ctx, A, vals, x, dscale, epi);
	}
}

}  // namespace fsg
