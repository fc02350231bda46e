// SpMV of a symmetric grid-stencil matrix from its diagonal and upper
// diagonals, rows addressed by their grid coordinates.
//
// The operator, the storage and the row loop are those of spmv_sym_kernel
// (the reference's compressed_ops::spmv row loop, flecsolve/matrices/
// seq.hh:177-193, on the symmetric storage): when the matrix is a 1-, 2- or
// 3-D grid stencil -- positive offsets 1, nx, nx ny and every row holding
// exactly its neighbours inside the grid (detected once at creation) -- a
// row's entries follow from its coordinates (i, j, k) alone, so no pattern
// id is read and no load waits on another.  A thread sums W = 16 / sizeof(V)
// consecutive rows of one grid line (nx a multiple of 4): each of the
// diagonal, the upper diagonals, the lower partners u_d[r - d] of the y and z
// offsets and x at r, r +- nx, r +- nx ny is one 16-byte load for all W rows;
// the two x neighbours along the line and u_1[r - 1] are single loads.  14
// loads for W rows instead of 14 per row, all independent.
//
// Each row sums the same products in the same (column) order as the CSR
// kernels, so results are identical bit for bit; boundary rows skip the
// neighbours outside the grid exactly as their CSR rows lack them.
//
// GEN: a grid stencil whose values are not symmetric (convection-diffusion)
// reads the general grid storage, where the lower diagonals l_d[r] =
// a(r, r - d) sit at row r after the upper ones: the lower partners become
// 16-byte loads at r like the upper diagonals, three more loads for W rows.
//
// Work: 256-thread CTAs, one W-row segment per thread and step (256 W rows a
// step); chunks of consecutive steps strided over a persistent grid, as in
// spmv_sym_kernel (neighbouring lines out of L1, neighbouring planes out of
// L2 inside the moving window of all CTAs).
#pragma once

namespace fsg {

template<class V>
struct CsrGrid {
	const V *__restrict__ S;  // (nsym + 1) x ld: diagonal, upper diagonals
	int64_t ld;
	int n;                    // rows = nx ny nz
	int nx, ny, nz;
	int K;                    // upper diagonals: 1 (line), 2 (plane), 3 (volume)
	int chunk;                // consecutive steps per chunk
};

constexpr int kGridThreads = 256;
constexpr int kGridChunk = 4;

template<class V, bool EXACT, bool GEN, class G, class Epi>
__global__ void __launch_bounds__(kGridThreads)
spmv_grid_kernel(CsrGrid<V> A, G g_in, Epi epi) {
	constexpr int NV = Epi::NV;
	constexpr int W = 16 / (int)sizeof(V);
	__shared__ double red[128];
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	G g = g_in;
	g.init();
	Acc<V, NV> acc;
	acc.init();
	const int nseg = A.n / W;
	const int nstep = (nseg + kGridThreads - 1) / kGridThreads;
	const int segs_per_line = A.nx / W;
	const int64_t nxy = (int64_t)A.nx * A.ny;
	const bool has_y = A.K >= 2, has_z = A.K >= 3;
	const V *__restrict__ D = A.S;
	const V *__restrict__ U1 = A.S + A.ld;
	const V *__restrict__ U2 = A.S + 2 * A.ld;
	const V *__restrict__ U3 = A.S + 3 * A.ld;
	// GEN: the lower diagonals after the K upper ones
	const V *__restrict__ L1 = A.S + (int64_t)(A.K + 1) * A.ld;
	const V *__restrict__ L2 = A.S + (int64_t)(A.K + 2) * A.ld;
	const V *__restrict__ L3 = A.S + (int64_t)(A.K + 3) * A.ld;
	for (int k = 0;; ++k) {
		const int chunk = (int)blockIdx.x + (k / A.chunk) * (int)gridDim.x;
		const int step = chunk * A.chunk + k % A.chunk;
		if (step >= nstep)
			break;
		const int s = step * kGridThreads + (int)threadIdx.x;
		if (s >= nseg)
			continue;
		const int line = s / segs_per_line;
		const int i0 = (s - line * segs_per_line) * W;
		const int r0 = s * W;
		const int jj = has_y ? line % A.ny : 0;
		const int kk = has_y ? line / A.ny : 0;
		const bool lo_x = i0 > 0, hi_x = i0 + W < A.nx;
		const bool lo_y = has_y && jj > 0, hi_y = has_y && jj < A.ny - 1;
		const bool lo_z = has_z && kk > 0, hi_z = has_z && kk < A.nz - 1;
		V d[W], u1[W], u2[W], u3[W], u2m[W], u3m[W], l1[W];
		V x[W], xmy[W], xpy[W], xmz[W], xpz[W];
		V u1m = V(0), xm1 = V(0), xp1 = V(0);
		ld_vec16(D + r0, d);
		ld_vec16(U1 + r0, u1);
		g.at_vec(r0, x);
		if constexpr (GEN)
			ld_vec16(L1 + r0, l1);
		if (lo_x) {
			if constexpr (!GEN)
				u1m = __ldg(U1 + r0 - 1);
			xm1 = g.at(r0 - 1);
		}
		if (hi_x)
			xp1 = g.at(r0 + W);
		if (has_y) {
			ld_vec16(U2 + r0, u2);
			if (lo_y) {
				if constexpr (GEN)
					ld_vec16(L2 + r0, u2m);
				else
					ld_vec16(U2 + r0 - A.nx, u2m);
				g.at_vec(r0 - A.nx, xmy);
			}
			if (hi_y)
				g.at_vec(r0 + A.nx, xpy);
		}
		if (has_z) {
			ld_vec16(U3 + r0, u3);
			if (lo_z) {
				if constexpr (GEN)
					ld_vec16(L3 + r0, u3m);
				else
					ld_vec16(U3 + (r0 - nxy), u3m);
				g.at_vec((int)(r0 - nxy), xmz);
			}
			if (hi_z)
				g.at_vec((int)(r0 + nxy), xpz);
		}
#pragma unroll
		for (int q = 0; q < W; ++q) {
			V sum = V(0);
			auto term = [&](V a, V xv) {
				if constexpr (EXACT)
					sum = add_rn(sum, mul_rn(a, xv));
				else
					sum = fma(a, xv, sum);
			};
			// column order: r - nx ny, r - nx, r - 1, r, r + 1, r + nx, r + nx ny
			if (lo_z)
				term(u3m[q], xmz[q]);
			if (lo_y)
				term(u2m[q], xmy[q]);
			if constexpr (GEN) {
				if (q > 0)
					term(l1[q], x[q - 1]);
				else if (lo_x)
					term(l1[0], xm1);
			}
			else {
				if (q > 0)
					term(u1[q - 1], x[q - 1]);
				else if (lo_x)
					term(u1m, xm1);
			}
			term(d[q], x[q]);
			if (q < W - 1)
				term(u1[q], x[q + 1]);
			else if (hi_x)
				term(u1[q], xp1);
			if (hi_y)
				term(u2[q], xpy[q]);
			if (hi_z)
				term(u3[q], xpz[q]);
			epi.row(r0 + q, sum, acc);
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

// The grid kernel reads x (and the gather's scale) 16 bytes at a time
template<class V>
inline bool grid_aligned(const Csr *A, const V *x, const V *dscale) {
	constexpr int W = 16 / (int)sizeof(V);
	return A->grid_nx % W == 0 && ((uintptr_t)x & 15) == 0 && ((uintptr_t)dscale & 15) == 0 &&
	       A->nrows < (int64_t)1 << 30;
}

template<class V>
inline const V *gen_vals(const Csr *A);
template<>
inline const double *gen_vals<double>(const Csr *A) { return A->gen64; }
template<>
inline const float *gen_vals<float>(const Csr *A) { return A->gen32; }

template<class V, bool EXACT, bool GEN, class G, class Epi>
static inline int launch_spmv_grid(Ctx *ctx, const Csr *A, const G &g, const Epi &epi) {
	static int per_sm = 0;  // resident CTAs per SM of this instantiation
	constexpr int W = 16 / (int)sizeof(V);
	auto kern = spmv_grid_kernel<V, EXACT, GEN, G, Epi>;
	if (per_sm == 0) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kGridThreads, 0) != cudaSuccess ||
		    nb < 1)
			nb = 1;
		per_sm = nb;
	}
	const int nseg = (int)(A->nrows / W);
	const int nstep = (nseg + kGridThreads - 1) / kGridThreads;
	const int resident = ctx->sms * std::min(per_sm, 8);
	const int chunk = nstep >= kGridChunk * resident ? kGridChunk : 1;
	const int nchunk = (nstep + chunk - 1) / chunk;
	const int grid = std::max(1, std::min(nchunk, resident));
	CsrGrid<V> d{GEN ? gen_vals<V>(A) : sym_vals<V>(A), A->sym_ld, (int)A->nrows, A->grid_nx,
	             A->grid_ny, A->grid_nz, A->nsym, chunk};
	return check_launch_rc(ctx, launch_pdl(ctx->stream, kern, grid, kGridThreads, 0, d, g, epi),
	                       GEN ? "spmv (grid stencil, general storage)"
	                           : "spmv (grid stencil, symmetric storage)");
}

}  // namespace fsg
