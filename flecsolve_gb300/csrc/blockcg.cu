// Block Jacobi-PCG (O'Leary, "The block conjugate gradient algorithm and
// related methods", LAA 29, 1980) for S = 16 right-hand sides of one
// operator.  No counterpart in the reference, whose solvers take one
// right-hand side per call (cg.hh:43-139 run 16 times).
//
// X, R, P, Q are N x S row-major (the S values of a row contiguous), so the
// SpMM reads A once for all S columns and gathers one S-value row of P per
// nonzero.  Per iteration:
//   Q = A P,  M = P^T Q                 (SpMM with the Gram product fused)
//   alpha = M^-1 G
//   X += P alpha,  R -= Q alpha,  Z = D^-1 R,  G' = Z^T R, ||R_j||
//   beta = G^-1 G',  P = Z + P beta,  G = G'
// Gram products: each CTA walks 16-row tiles; thread (i, j) of the 256 sums
// P[r][i] Q[r][j] over the tile's rows, adds that tile sum to its running
// sum, and the per-CTA sums are folded in CTA order by the last CTA
// (deterministic).
//
// Two precisions share the kernels (template V):
//  * FP64 (fs_block_cg_solve): every vector and the matrix in FP64.  On this
//    GPU the FP64 pipe issues about 2 FMA per clock per SM, and an iteration
//    is ~5 N S^2 FMA, so this variant is bound by FP64 issue, not by HBM.
//  * FP32 recurrences with FP64 residual replacement
//    (fs_block_cg_solve_mixed): P, Q, R and a correction to X in FP32, FP32
//    matrix values, tile sums accumulated with compensated (two-sum) FP32
//    additions.  When every unconverged column's recurrence residual has
//    dropped by `delta` since the last replacement, or one of them is below
//    its tolerance, or at maxiter, the correction is folded into the FP64 X
//    and R is replaced by the FP64 residual B - A X (FP64 values).  A column
//    converges only on that FP64 residual (the reference's stopping test,
//    cg.hh:55-60, per column).  The search directions are kept across a
//    replacement (reliable updates, van der Vorst & Ye 2000).
// Columns that converge keep iterating inside the block until all have; the
// block stops when every column has converged or at maxiter.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <type_traits>

#include "solver.cuh"

namespace fsg {
namespace {

constexpr int kS = 16;     // right-hand sides per block
constexpr int kTile = 16;  // rows per tile (kTile * kS = 256 threads)
constexpr int BCG_REPLACE = 1;

struct BcgState {
	double G[kS * kS], Gn[kS * kS], M[kS * kS], alpha[kS * kS], beta[kS * kS];
	double bnorm[kS], rnorm[kS], res0[kS], rlast[kS];
	int conv_iter[kS];
	int iter, done, status, flags, replacements;
};

// running sums: plain FP64, or compensated FP32 (Knuth's two-sum on every
// addition; value = hi + lo)
template<class V>
struct BAcc;
template<>
struct BAcc<double> {
	double s = 0.0;
	__device__ void add(double v) { s += v; }
	__device__ double get() const { return s; }
};
template<>
struct BAcc<float> {
	float hi = 0.f, lo = 0.f;
	__device__ void add(float v) {
		const float s = hi + v;
		const float bp = s - hi;
		lo += (hi - (s - bp)) + (v - bp);
		hi = s;
	}
	__device__ double get() const { return (double)hi + (double)lo; }
};

// sum over the tile's rows of a[rr][i] * b[rr][j]
template<class V>
__device__ __forceinline__ V tile_dot(const V (*a)[kS], const V (*b)[kS], int i, int j) {
	V t = 0;
#pragma unroll
	for (int rr = 0; rr < kTile; ++rr)
		t = fma(a[rr][i], b[rr][j], t);
	return t;
}

__device__ __forceinline__ bool bcg_skip(const BcgState *st) {
	return st->done || (st->flags & BCG_REPLACE);
}

// x = A^-1 B for the s x s matrix A (row-major), s right-hand sides in B
// (row-major, overwritten with the solution): Gaussian elimination with
// partial pivoting.  Returns false on a zero pivot.  Single thread.
__device__ bool small_solve(double *A, double *B) {
	for (int k = 0; k < kS; ++k) {
		int p = k;
		double m = fabs(A[k * kS + k]);
		for (int i = k + 1; i < kS; ++i)
			if (fabs(A[i * kS + k]) > m) {
				m = fabs(A[i * kS + k]);
				p = i;
			}
		if (!(m > 0.0))
			return false;
		if (p != k) {
			for (int j = 0; j < kS; ++j) {
				double t = A[k * kS + j];
				A[k * kS + j] = A[p * kS + j];
				A[p * kS + j] = t;
				t = B[k * kS + j];
				B[k * kS + j] = B[p * kS + j];
				B[p * kS + j] = t;
			}
		}
		for (int i = k + 1; i < kS; ++i) {
			const double f = A[i * kS + k] / A[k * kS + k];
			for (int j = k; j < kS; ++j)
				A[i * kS + j] -= f * A[k * kS + j];
			for (int j = 0; j < kS; ++j)
				B[i * kS + j] -= f * B[k * kS + j];
		}
	}
	for (int k = kS - 1; k >= 0; --k)
		for (int j = 0; j < kS; ++j) {
			double s = B[k * kS + j];
			for (int i = k + 1; i < kS; ++i)
				s -= A[k * kS + i] * B[i * kS + j];
			B[k * kS + j] = s / A[k * kS + k];
		}
	return true;
}

// beta = G^-1 G', G = G' (single thread); false on breakdown
__device__ bool form_beta(BcgState *st) {
	double Gc[kS * kS];
	for (int i = 0; i < kS * kS; ++i) {
		Gc[i] = st->G[i];
		st->beta[i] = st->Gn[i];
	}
	const bool ok = small_solve(Gc, st->beta);
	for (int i = 0; i < kS * kS; ++i)
		st->G[i] = st->Gn[i];
	return ok;
}

// Q = A P and the CTA's part of M = P^T Q; the last CTA forms alpha = M^-1 G
template<class V>
__global__ void __launch_bounds__(256)
k_bcg_spmm(int n, const int *__restrict__ rp, const int *__restrict__ col,
           const V *__restrict__ val, const V *__restrict__ P, V *__restrict__ Q, BcgState *st,
           double *part, unsigned *counter) {
	__shared__ V sp[kTile][kS], sq[kTile][kS];
	if (bcg_skip(st))
		return;
	const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
	const int ntiles = (n + kTile - 1) / kTile;
	BAcc<V> m;
	for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const int r = t * kTile + tr;
		V q = 0, p = 0;
		if (r < n) {
			for (int k = rp[r]; k < rp[r + 1]; ++k)
				q = fma(val[k], P[(size_t)col[k] * kS + tj], q);
			Q[(size_t)r * kS + tj] = q;
			p = P[(size_t)r * kS + tj];
		}
		sp[tr][tj] = p;
		sq[tr][tj] = q;
		__syncthreads();
		m.add(tile_dot<V>(sp, sq, tr, tj));
		__syncthreads();
	}
	part[(size_t)blockIdx.x * 256 + threadIdx.x] = m.get();
	if (last_block(counter)) {
		double s = 0.0;
		for (unsigned b = 0; b < gridDim.x; ++b)
			s += __ldcg(part + (size_t)b * 256 + threadIdx.x);
		st->M[threadIdx.x] = s;
		__syncthreads();
		if (threadIdx.x == 0) {
			double Mc[kS * kS];
			for (int i = 0; i < kS * kS; ++i) {
				Mc[i] = st->M[i];
				st->alpha[i] = st->G[i];
			}
			if (!small_solve(Mc, st->alpha)) {
				st->done = 1;
				st->status = FS_DIVERGED_BREAKDOWN;
			}
			*counter = 0;
		}
	}
}

// X += P alpha, R -= Q alpha, Z = D^-1 R; G' = Z^T R and ||R_j||^2 parts.
// The last CTA counts the iteration and then
//  * FP64 (delta <= 0): marks the columns below tolerance, stops when all
//    are, else forms beta;
//  * mixed (delta > 0): requests a residual replacement when every
//    unconverged column has dropped by delta since the last one, or one is
//    below tolerance, or at maxiter; else forms beta.
template<class V>
__global__ void __launch_bounds__(256)
k_bcg_update(int n, V *__restrict__ X, const V *__restrict__ P, V *__restrict__ R,
             const V *__restrict__ Q, const V *__restrict__ dinv, BcgState *st, double *part,
             double *part2, unsigned *counter, double tolf, int maxiter, double delta) {
	__shared__ V sa[kS * kS], sp[kTile][kS], sq[kTile][kS], sr[kTile][kS], sz[kTile][kS];
	__shared__ double cn[kTile][kS];
	if (bcg_skip(st))
		return;
	sa[threadIdx.x] = (V)st->alpha[threadIdx.x];
	__syncthreads();
	const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
	const int ntiles = (n + kTile - 1) / kTile;
	BAcc<V> g, nr;
	for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const int r = t * kTile + tr;
		sp[tr][tj] = r < n ? P[(size_t)r * kS + tj] : V(0);
		sq[tr][tj] = r < n ? Q[(size_t)r * kS + tj] : V(0);
		__syncthreads();
		V rv = 0, z = 0;
		if (r < n) {
			V x = X[(size_t)r * kS + tj];
			rv = R[(size_t)r * kS + tj];
#pragma unroll
			for (int i = 0; i < kS; ++i) {
				x = fma(sp[tr][i], sa[i * kS + tj], x);
				rv = fma(-sq[tr][i], sa[i * kS + tj], rv);
			}
			X[(size_t)r * kS + tj] = x;
			R[(size_t)r * kS + tj] = rv;
			z = dinv ? dinv[r] * rv : rv;
			nr.add(rv * rv);
		}
		sr[tr][tj] = rv;
		sz[tr][tj] = z;
		__syncthreads();
		g.add(tile_dot<V>(sz, sr, tr, tj));
		__syncthreads();
	}
	part[(size_t)blockIdx.x * 256 + threadIdx.x] = g.get();
	// column norms: fold the 16 row-threads of each column in the block first
	cn[tr][tj] = nr.get();
	__syncthreads();
	if (threadIdx.x < kS) {
		double c = 0.0;
		for (int rr = 0; rr < kTile; ++rr)
			c += cn[rr][threadIdx.x];
		part2[(size_t)blockIdx.x * kS + threadIdx.x] = c;
	}
	if (last_block(counter)) {
		double s = 0.0;
		for (unsigned b = 0; b < gridDim.x; ++b)
			s += __ldcg(part + (size_t)b * 256 + threadIdx.x);
		st->Gn[threadIdx.x] = s;
		if (threadIdx.x < kS) {
			double c = 0.0;
			for (unsigned b = 0; b < gridDim.x; ++b)
				c += __ldcg(part2 + (size_t)b * kS + threadIdx.x);
			st->rnorm[threadIdx.x] = sqrt(c);
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			const int it = st->iter + 1;
			st->iter = it;
			bool finite = true;
			for (int j = 0; j < kS; ++j)
				finite = finite && isfinite(st->rnorm[j]);
			if (delta <= 0.0) {
				bool all = true;
				for (int j = 0; j < kS; ++j) {
					if (st->conv_iter[j] == 0 && st->rnorm[j] < tolf * st->bnorm[j])
						st->conv_iter[j] = it;
					all = all && st->conv_iter[j] != 0;
				}
				if (all) {
					st->done = 1;
					st->status = FS_CONVERGED_RTOL;
				}
				else if (!finite) {
					st->done = 1;
					st->status = FS_DIVERGED_BREAKDOWN;
				}
				else if (it >= maxiter) {
					st->done = 1;
					st->status = FS_DIVERGED_ITERS;
				}
				else if (!form_beta(st)) {
					st->done = 1;
					st->status = FS_DIVERGED_BREAKDOWN;
				}
			}
			else {
				bool replace = it >= maxiter || !finite;
				double worst = 0.0;
				for (int j = 0; j < kS; ++j) {
					if (st->conv_iter[j] != 0)
						continue;
					if (st->rnorm[j] < tolf * st->bnorm[j])
						replace = true;
					const double q = st->rlast[j] > 0.0 ? st->rnorm[j] / st->rlast[j] : 0.0;
					worst = q > worst ? q : worst;
				}
				if (replace || worst < delta)
					st->flags |= BCG_REPLACE;
				else if (!form_beta(st)) {
					st->done = 1;
					st->status = FS_DIVERGED_BREAKDOWN;
				}
			}
			*counter = 0;
		}
	}
}

// P = Z + P beta (Z = D^-1 R)
template<class V>
__global__ void __launch_bounds__(256)
k_bcg_dir(int n, V *__restrict__ P, const V *__restrict__ R, const V *__restrict__ dinv,
          const BcgState *st) {
	__shared__ V sb[kS * kS], sp[kTile][kS];
	if (bcg_skip(st))
		return;
	sb[threadIdx.x] = (V)st->beta[threadIdx.x];
	const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
	const int ntiles = (n + kTile - 1) / kTile;
	for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const int r = t * kTile + tr;
		__syncthreads();
		sp[tr][tj] = r < n ? P[(size_t)r * kS + tj] : V(0);
		__syncthreads();
		if (r < n) {
			V p = (dinv ? dinv[r] : V(1)) * R[(size_t)r * kS + tj];
#pragma unroll
			for (int i = 0; i < kS; ++i)
				p = fma(sp[tr][i], sb[i * kS + tj], p);
			P[(size_t)r * kS + tj] = p;
		}
	}
}

// R = B - A X (FP64 values; X64 = 0 first for a zero guess), Rv = (V) R,
// P = Z = D^-1 Rv, G = Z^T Rv, ||B_j||, ||R_j||.  Xc, when given, is the FP32
// correction of the mixed variant and is cleared.
template<class V>
__global__ void __launch_bounds__(256)
k_bcg_start(int n, const int *__restrict__ rp, const int *__restrict__ col,
            const double *__restrict__ val, const double *__restrict__ B, double *__restrict__ X,
            V *__restrict__ Xc, V *__restrict__ R, V *__restrict__ P, const V *__restrict__ dinv,
            int zero_guess, BcgState *st, double *part, double *part2, unsigned *counter) {
	__shared__ V sr[kTile][kS], sz[kTile][kS];
	__shared__ double cb[kTile][kS], cr[kTile][kS];
	const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
	const int ntiles = (n + kTile - 1) / kTile;
	BAcc<V> g;
	double nb = 0.0, nr = 0.0;
	for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const int r = t * kTile + tr;
		V rv = 0, z = 0;
		if (r < n) {
			const double bv = B[(size_t)r * kS + tj];
			double ax = 0.0;
			if (zero_guess)
				X[(size_t)r * kS + tj] = 0.0;
			else
				for (int k = rp[r]; k < rp[r + 1]; ++k)
					ax = fma(val[k], X[(size_t)col[k] * kS + tj], ax);
			const double r64 = bv - ax;
			if (Xc)
				Xc[(size_t)r * kS + tj] = V(0);
			rv = (V)r64;
			R[(size_t)r * kS + tj] = rv;
			z = dinv ? dinv[r] * rv : rv;
			P[(size_t)r * kS + tj] = z;
			nb = fma(bv, bv, nb);
			nr = fma(r64, r64, nr);
		}
		sr[tr][tj] = rv;
		sz[tr][tj] = z;
		__syncthreads();
		g.add(tile_dot<V>(sz, sr, tr, tj));
		__syncthreads();
	}
	part[(size_t)blockIdx.x * 256 + threadIdx.x] = g.get();
	cb[tr][tj] = nb;
	cr[tr][tj] = nr;
	__syncthreads();
	if (threadIdx.x < kS) {
		double c1 = 0.0, c2 = 0.0;
		for (int rr = 0; rr < kTile; ++rr) {
			c1 += cb[rr][threadIdx.x];
			c2 += cr[rr][threadIdx.x];
		}
		part2[(size_t)blockIdx.x * 2 * kS + threadIdx.x] = c1;
		part2[(size_t)blockIdx.x * 2 * kS + kS + threadIdx.x] = c2;
	}
	if (last_block(counter)) {
		double s = 0.0;
		for (unsigned b = 0; b < gridDim.x; ++b)
			s += __ldcg(part + (size_t)b * 256 + threadIdx.x);
		st->G[threadIdx.x] = s;
		if (threadIdx.x < kS) {
			double c1 = 0.0, c2 = 0.0;
			for (unsigned b = 0; b < gridDim.x; ++b) {
				c1 += __ldcg(part2 + (size_t)b * 2 * kS + threadIdx.x);
				c2 += __ldcg(part2 + (size_t)b * 2 * kS + kS + threadIdx.x);
			}
			const double bn = sqrt(c1);
			st->bnorm[threadIdx.x] = bn == 0.0 ? 1.0 : bn;
			st->rnorm[threadIdx.x] = sqrt(c2);
			st->res0[threadIdx.x] = sqrt(c2);
			st->rlast[threadIdx.x] = sqrt(c2);
			st->conv_iter[threadIdx.x] = 0;
		}
		if (threadIdx.x == 0) {
			st->iter = 0;
			st->done = 0;
			st->status = FS_STATUS_UNKNOWN;
			st->flags = 0;
			st->replacements = 0;
			*counter = 0;
		}
	}
}

// mixed: X64 += Xc, Xc = 0
__global__ void k_bcg_fold(size_t m, double *__restrict__ X, float *__restrict__ Xc) {
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m;
	     i += (size_t)gridDim.x * blockDim.x) {
		X[i] += (double)Xc[i];
		Xc[i] = 0.f;
	}
}

// mixed: R = (float)(B - A X) with the FP64 values, ||R_j|| in FP64,
// G' = Z^T R; the last CTA decides convergence per column on the FP64
// residual, resets the replacement reference levels and forms beta
__global__ void __launch_bounds__(256)
k_bcg_true_res(int n, const int *__restrict__ rp, const int *__restrict__ col,
               const double *__restrict__ val, const double *__restrict__ B,
               const double *__restrict__ X, float *__restrict__ R, const float *__restrict__ dinv,
               BcgState *st, double *part, double *part2, unsigned *counter, double tolf,
               int maxiter) {
	__shared__ float sr[kTile][kS], sz[kTile][kS];
	__shared__ double cr[kTile][kS];
	const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
	const int ntiles = (n + kTile - 1) / kTile;
	BAcc<float> g;
	double nr = 0.0;
	for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const int r = t * kTile + tr;
		float rv = 0.f, z = 0.f;
		if (r < n) {
			double ax = 0.0;
			for (int k = rp[r]; k < rp[r + 1]; ++k)
				ax = fma(val[k], X[(size_t)col[k] * kS + tj], ax);
			const double r64 = B[(size_t)r * kS + tj] - ax;
			rv = (float)r64;
			R[(size_t)r * kS + tj] = rv;
			z = dinv ? dinv[r] * rv : rv;
			nr = fma(r64, r64, nr);
		}
		sr[tr][tj] = rv;
		sz[tr][tj] = z;
		__syncthreads();
		g.add(tile_dot<float>(sz, sr, tr, tj));
		__syncthreads();
	}
	part[(size_t)blockIdx.x * 256 + threadIdx.x] = g.get();
	cr[tr][tj] = nr;
	__syncthreads();
	if (threadIdx.x < kS) {
		double c = 0.0;
		for (int rr = 0; rr < kTile; ++rr)
			c += cr[rr][threadIdx.x];
		part2[(size_t)blockIdx.x * kS + threadIdx.x] = c;
	}
	if (last_block(counter)) {
		double s = 0.0;
		for (unsigned b = 0; b < gridDim.x; ++b)
			s += __ldcg(part + (size_t)b * 256 + threadIdx.x);
		st->Gn[threadIdx.x] = s;
		if (threadIdx.x < kS) {
			double c = 0.0;
			for (unsigned b = 0; b < gridDim.x; ++b)
				c += __ldcg(part2 + (size_t)b * kS + threadIdx.x);
			st->rnorm[threadIdx.x] = sqrt(c);
			st->rlast[threadIdx.x] = sqrt(c);
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			const int it = st->iter;
			bool all = true, finite = true;
			for (int j = 0; j < kS; ++j) {
				finite = finite && isfinite(st->rnorm[j]);
				if (st->conv_iter[j] == 0 && st->rnorm[j] < tolf * st->bnorm[j])
					st->conv_iter[j] = it > 0 ? it : 1;
				all = all && st->conv_iter[j] != 0;
			}
			st->replacements += 1;
			st->flags &= ~BCG_REPLACE;
			if (all) {
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
			}
			else if (!finite) {
				st->done = 1;
				st->status = FS_DIVERGED_BREAKDOWN;
			}
			else if (it >= maxiter) {
				st->done = 1;
				st->status = FS_DIVERGED_ITERS;
			}
			else if (!form_beta(st)) {
				st->done = 1;
				st->status = FS_DIVERGED_BREAKDOWN;
			}
			*counter = 0;
		}
	}
}

struct BcgPlan {
	BcgState *st = nullptr, *hst = nullptr;
	void *work = nullptr;       // P, Q, R (and the FP32 X correction)
	double *part = nullptr;     // G partials (grid x 256) + norm partials
	unsigned *counter = nullptr;
	int64_t n = 0;
};
std::map<std::pair<const Csr *, bool>, BcgPlan> g_bcg;

template<class V>
int block_cg_run(Ctx *ctx, const fs_krylov_settings *s, Csr *A, bool jac, Vec *B, Vec *X,
                 fs_solve_info *infos) {
	constexpr bool mixed = std::is_same<V, float>::value;
	const int64_t n = A->nrows;
	if (jac)
		FS_TRY(ensure_dinv(A));
	if (mixed)
		FS_TRY(ensure_val32(A));
	BcgPlan &p = g_bcg[std::make_pair((const Csr *)A, mixed)];
	const int G = std::max(1, std::min(ctx->sms * 8, (int)((n + kTile - 1) / kTile)));
	const size_t m = (size_t)n * kS;
	if (p.n != n) {
		if (p.work) {
			cudaStreamSynchronize(ctx->stream);
			cudaFree(p.work);
			cudaFree(p.part);
			cudaFree(p.counter);
			cudaFree(p.st);
			cudaFreeHost(p.hst);
			p = BcgPlan();
		}
		FS_CUDA_TRY(ctx, cudaMalloc(&p.work, sizeof(V) * (mixed ? 4 : 3) * m));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.part, sizeof(double) * (size_t)ctx->sms * 8 * (256 + 2 * kS)));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.counter, 64));
		FS_CUDA_TRY(ctx, cudaMemset(p.counter, 0, 64));
		FS_CUDA_TRY(ctx, fence_setup_copies());
		FS_CUDA_TRY(ctx, cudaMalloc(&p.st, sizeof(BcgState)));
		FS_CUDA_TRY(ctx, cudaMallocHost(&p.hst, sizeof(BcgState)));
		p.n = n;
	}
	V *Pm = (V *)p.work, *Qm = Pm + m, *R = Pm + 2 * m;
	V *Xc = mixed ? Pm + 3 * m : nullptr;
	double *part = p.part, *part2 = p.part + (size_t)ctx->sms * 8 * 256;
	const V *dinv = nullptr;
	if (jac)
		dinv = mixed ? (const V *)A->dinv32 : (const V *)A->dinv;
	const V *val = mixed ? (const V *)A->val32 : (const V *)A->val;
	const double *b = (const double *)B->d;
	double *x = (double *)X->d;
	V *xv = mixed ? Xc : (V *)x;
	k_bcg_start<V><<<G, 256, 0, ctx->stream>>>((int)n, A->rowptr, A->col, A->val, b, x, Xc, R, Pm,
	                                           dinv, s->base.use_zero_guess ? 1 : 0, p.st, part,
	                                           part2, p.counter);
	FS_TRY(check_launch(ctx, "block cg start"));
	const double tolf = (double)s->base.rtol;
	const int maxiter = s->base.maxiter;
	const int k = s->k_readback > 0 ? s->k_readback : 16;
	const double delta = mixed ? (s->inner_rtol > 0 ? s->inner_rtol : 0.1) : 0.0;
	auto read_back = [&]() -> int {
		FS_CUDA_TRY(ctx, cudaMemcpyAsync(p.hst, p.st, sizeof(BcgState), cudaMemcpyDeviceToHost,
		                                 ctx->stream));
		FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
		return FS_OK;
	};
	FS_TRY(read_back());
	while (!p.hst->done) {
		for (int j = 0; j < k; ++j) {
			k_bcg_spmm<V><<<G, 256, 0, ctx->stream>>>((int)n, A->rowptr, A->col, val, Pm, Qm, p.st,
			                                          part, p.counter);
			FS_TRY(check_launch(ctx, "block cg spmm"));
			k_bcg_update<V><<<G, 256, 0, ctx->stream>>>((int)n, xv, Pm, R, Qm, dinv, p.st, part,
			                                            part2, p.counter, tolf, maxiter, delta);
			FS_TRY(check_launch(ctx, "block cg update"));
			k_bcg_dir<V><<<G, 256, 0, ctx->stream>>>((int)n, Pm, R, dinv, p.st);
			FS_TRY(check_launch(ctx, "block cg direction"));
		}
		FS_TRY(read_back());
		if (mixed && !p.hst->done && (p.hst->flags & BCG_REPLACE)) {
			k_bcg_fold<<<grid_for(ctx, (int64_t)m, 256, 8), 256, 0, ctx->stream>>>(m, x, (float *)Xc);
			FS_TRY(check_launch(ctx, "block cg fold"));
			k_bcg_true_res<<<G, 256, 0, ctx->stream>>>((int)n, A->rowptr, A->col, A->val, b, x,
			                                           (float *)R, (const float *)dinv, p.st, part,
			                                           part2, p.counter, tolf, maxiter);
			FS_TRY(check_launch(ctx, "block cg true residual"));
			k_bcg_dir<V><<<G, 256, 0, ctx->stream>>>((int)n, Pm, R, dinv, p.st);
			FS_TRY(check_launch(ctx, "block cg direction"));
			FS_TRY(read_back());
		}
		if (!p.hst->done && p.hst->iter >= maxiter && !(p.hst->flags & BCG_REPLACE))
			break;
	}
	if (mixed && !(p.hst->done && p.hst->status == FS_CONVERGED_RTOL)) {
		// a stop without a final replacement (breakdown): keep the progress
		k_bcg_fold<<<grid_for(ctx, (int64_t)m, 256, 8), 256, 0, ctx->stream>>>(m, x, (float *)Xc);
		FS_TRY(check_launch(ctx, "block cg fold"));
		FS_TRY(read_back());
	}
	const BcgState &hs = *p.hst;
	for (int j = 0; j < kS; ++j) {
		fs_solve_info &inf = infos[j];
		memset(&inf, 0, sizeof inf);
		inf.status = hs.conv_iter[j] ? FS_CONVERGED_RTOL
		                             : (hs.status == FS_DIVERGED_BREAKDOWN ? FS_DIVERGED_BREAKDOWN
		                                                                   : FS_DIVERGED_ITERS);
		inf.iters = hs.conv_iter[j];
		inf.restarts = hs.iter;  // block iterations run
		inf.res_norm_initial = (float)hs.res0[j];
		inf.res_norm_final = (float)hs.rnorm[j];
		inf.rhs_norm = (float)hs.bnorm[j];
	}
	return FS_OK;
}

int block_cg_entry(fs_ctx h, const fs_krylov_settings *s, fs_csr Ah, const fs_precond *Pc, int nrhs,
                   fs_vec bh, fs_vec xh, fs_solve_info *infos, bool mixed) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Csr *A = reinterpret_cast<Csr *>(Ah);
	Vec *B = reinterpret_cast<Vec *>(bh), *X = reinterpret_cast<Vec *>(xh);
	if (!ok_ctx(ctx) || !ok_csr(A) || !ok_vec(B) || !ok_vec(X) || !s || !infos)
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "block_cg_entry"));
	if (nrhs != kS)
		return set_err(ctx, FS_ERR_UNSUPPORTED, "block CG: this build takes %d right-hand sides", kS);
	const int64_t n = A->nrows;
	if (A->nrows != A->ncols || B->n != n * kS || X->n != n * kS || B->dtype != FS_F64 ||
	    X->dtype != FS_F64)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "block CG: B and X hold N x %d FP64 row-major", kS);
	if (n == 0)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "block CG: empty operator");
	const bool jac = Pc && Pc->kind == FS_PRECOND_JACOBI;
	if (Pc && Pc->kind != FS_PRECOND_NONE && !jac)
		return set_err(ctx, FS_ERR_UNSUPPORTED, "block CG: identity or Jacobi preconditioner");
	if (s->base.maxiter < 1)
		return set_err(ctx, FS_ERR_INVALID_ARG, "block CG: maxiter must be positive");
	cudaSetDevice(ctx->device);
	return mixed ? block_cg_run<float>(ctx, s, A, jac, B, X, infos)
	             : block_cg_run<double>(ctx, s, A, jac, B, X, infos);
}

}  // namespace
}  // namespace fsg

extern "C" FS_API int fs_block_cg_solve(fs_ctx h, const fs_krylov_settings *s, fs_csr A,
                                        const fs_precond *P, int nrhs, fs_vec B, fs_vec X,
                                        fs_solve_info *infos) {
	return fsg::block_cg_entry(h, s, A, P, nrhs, B, X, infos, false);
}

extern "C" FS_API int fs_block_cg_solve_mixed(fs_ctx h, const fs_krylov_settings *s, fs_csr A,
                                              const fs_precond *P, int nrhs, fs_vec B, fs_vec X,
                                              fs_solve_info *infos) {
	return fsg::block_cg_entry(h, s, A, P, nrhs, B, X, infos, true);
}
