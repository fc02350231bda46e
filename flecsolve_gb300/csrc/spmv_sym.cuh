// Row-pattern SpMV of a symmetric matrix from its diagonal and upper
// diagonals.
//
// Same operator and row loop as spmv_rb_kernel (the reference's
// compressed_ops::spmv row loop, flecsolve/matrices/seq.hh:177-193).  When
// a row-pattern matrix is symmetric bit for bit (a_ij and a_ji the same
// double; the finite-volume diffusion operators are), every off-diagonal
// value is stored twice in CSR.  This format keeps the diagonal and, for each
// positive column offset d of the patterns, the "upper diagonal" u_d[r] =
// a(r, r + d); the entry a(r, r - d) of the lower triangle is u_d[r - d].  A
// 7-point operator then reads 4 values per row instead of 7, and no indices
// besides the one-byte pattern id.
//
// One thread per row of a 256-row tile, tiles strided over a persistent grid
// (the x and u values of neighbouring grid lines and planes are re-read out
// of L1/L2).  Every load of a warp is one contiguous segment, so there is
// nothing to stage.  Per pattern
// a table gives, for each entry in column order, the offset of its value
// from r in the storage (the diagonal, an upper diagonal at r, or an upper
// diagonal at r - d) and of its column from r, so a row costs two adds, two
// loads and one multiply-add per nonzero and sums the same products in the
// same order as the CSR kernels: the results are identical bit for bit.  x
// comes from the same gather policies as the row-pattern kernel
// (spmv_pat.cuh).
#pragma once

namespace fsg {

template<class V>
struct CsrSym {
	const V *__restrict__ S;                  // (nsym + 1) x ld: diagonal, upper diagonals
	const unsigned char *__restrict__ pid;
	const int2 *__restrict__ tab;             // npat x kPatW {value offset, column offset}
	const unsigned char *__restrict__ plen;
	int n, npat;
	int chunk;  // consecutive steps per chunk (1 .. kSymChunk)
};

constexpr int kSymThreads = 256;
// rows per thread and step: two for float (64 registers, 4 CTAs per SM), one
// for double (two would need ~100 registers)
template<class V>
constexpr int kSymRows = sizeof(V) == 4 ? 2 : 1;
constexpr int kSymChunk = 4;  // consecutive steps per chunk on large operators

template<class V, bool EXACT, class G, class Epi>
__global__ void __launch_bounds__(kSymThreads)
spmv_sym_kernel(CsrSym<V> A, G g_in, Epi epi) {
	constexpr int NV = Epi::NV;
	constexpr int kSymRows = fsg::kSymRows<V>;
	extern __shared__ __align__(16) int2 tab[];  // npat x kPatW
	__shared__ unsigned char plen[kMaxPat];
	__shared__ double red[128];
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	G g = g_in;
	g.init();
	for (int i = threadIdx.x; i < A.npat * kPatW; i += blockDim.x)
		tab[i] = A.tab[i];
	for (int i = threadIdx.x; i < A.npat; i += blockDim.x)
		plen[i] = A.plen[i];
	__syncthreads();
	Acc<V, NV> acc;
	acc.init();
	// kSymRows adjacent tiles per step; A.chunk consecutive steps per chunk
	// (the x and u values of neighbouring grid lines are then re-read out of
	// L1); chunks strided over the grid, so all CTAs work inside one moving
	// window of the vectors (few pages in flight, neighbouring planes in L2).
	// A thread sums one row of each tile; the pattern ids of its next step
	// are loaded before this step's values.
	const int ntile = (A.n + kSymThreads - 1) / kSymThreads;
	const int nstep = (ntile + kSymRows - 1) / kSymRows;
	auto step_tile = [&](int k) -> int {  // first tile of this CTA's k-th step
		const int chunk = (int)blockIdx.x + (k / A.chunk) * (int)gridDim.x;
		return (chunk * A.chunk + k % A.chunk) * kSymRows;
	};
	auto pid_at = [&](int t) -> int {
		const int r = t * kSymThreads + threadIdx.x;
		return t < ntile && r < A.n ? (int)ld_stream(A.pid + r) : -1;
	};
	int pnext[kSymRows];
#pragma unroll
	for (int u = 0; u < kSymRows; ++u)
		pnext[u] = pid_at(step_tile(0) + u);
	for (int k = 0; step_tile(k) < nstep * kSymRows; ++k) {
		const int t = step_tile(k);
		int pc[kSymRows];
		const int tn = step_tile(k + 1);
#pragma unroll
		for (int u = 0; u < kSymRows; ++u) {
			pc[u] = pnext[u];
			pnext[u] = pid_at(tn + u);
		}
		V a[kSymRows][kPatW], xv[kSymRows][kPatW];
		int len[kSymRows];
#pragma unroll
		for (int u = 0; u < kSymRows; ++u) {
			const int r = (t + u) * kSymThreads + threadIdx.x;
			len[u] = pc[u] >= 0 ? plen[pc[u]] : 0;
			if (len[u] > 0) {
				// entry j: value S[r + vo[j]], column r + xo[j]
				const int4 *tp = reinterpret_cast<const int4 *>(tab + pc[u] * kPatW);
				const int4 q0 = tp[0], q1 = tp[1], q2 = tp[2], q3 = tp[3];
				const int vo[kPatW] = {q0.x, q0.z, q1.x, q1.z, q2.x, q2.z, q3.x, q3.z};
				const int xo[kPatW] = {q0.y, q0.w, q1.y, q1.w, q2.y, q2.w, q3.y, q3.w};
#pragma unroll
				for (int j = 0; j < kPatW; ++j)
					if (j < len[u]) {
						a[u][j] = ld_stream(A.S + (r + vo[j]));
						xv[u][j] = g.at_stream(r + xo[j]);
					}
			}
		}
#pragma unroll
		for (int u = 0; u < kSymRows; ++u) {
			const int r = (t + u) * kSymThreads + threadIdx.x;
			if (pc[u] < 0)
				continue;
			V sum = V(0);
#pragma unroll
			for (int j = 0; j < kPatW; ++j)
				if (j < len[u]) {
					if constexpr (EXACT)
						sum = add_rn(sum, mul_rn(a[u][j], xv[u][j]));
					else
						sum = fma(a[u][j], xv[u][j], sum);
				}
			epi.row(r, sum, acc);
		}
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

template<class V>
inline const V *sym_vals(const Csr *A);
template<>
inline const double *sym_vals<double>(const Csr *A) { return A->sym64; }
template<>
inline const float *sym_vals<float>(const Csr *A) { return A->sym32; }

template<class V, bool EXACT, class G, class Epi>
static inline int launch_spmv_sym(Ctx *ctx, const Csr *A, const G &g, const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	constexpr size_t smem = sizeof(int2) * kMaxPat * kPatW;
	auto kern = spmv_sym_kernel<V, EXACT, G, Epi>;
	if (per_sm == 0) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kSymThreads, smem) != cudaSuccess ||
		    nb < 1)
			nb = 1;
		per_sm = nb;
	}
	// chunks of consecutive steps only on operators with at least kSymChunk
	// steps per resident CTA; a smaller operator keeps one step per chunk
	// (and its CTA grouping of the fused reductions)
	const int nstep = (int)((A->nrows + kSymThreads * kSymRows<V> - 1) / (kSymThreads * kSymRows<V>));
	const int resident = ctx->sms * std::min(per_sm, 8);
	const int chunk = nstep >= kSymChunk * resident ? kSymChunk : 1;
	const int nchunk = (nstep + chunk - 1) / chunk;
	const int grid = std::max(1, std::min(nchunk, resident));
	CsrSym<V> d{sym_vals<V>(A), A->pid, A->stab, A->plen, (int)A->nrows, A->npat, chunk};
	return check_launch_rc(ctx, launch_pdl(ctx->stream, kern, grid, kSymThreads, smem, d, g, epi),
	                       "spmv (symmetric row patterns)");
}

}  // namespace fsg
