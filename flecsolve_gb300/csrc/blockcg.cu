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
// Gram products: each CTA walks 64-row steps; thread (g, a, b) of the 256
// accumulates the 4 x 4 block [4a, 4a+4) x [4b, 4b+4) over the step's rows
// g, g + 16, g + 32, g + 48 (register blocking: 16-byte loads, 16 FMAs per
// pair of loads), adds that step sum to its running sum, and the per-CTA
// sums are folded in a fixed two-level order (groups of 32 CTAs, then the
// groups), so the result is deterministic for a given grid.
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

__device__ __forceinline__ bool bcg_skip(const BcgState *st) {
	return st->done || (st->flags & BCG_REPLACE);
}

// sum over a 16-row tile of a[rr][i] * b[rr][j] (start and replacement
// kernels)
template<class V>
__device__ __forceinline__ V tile_dot(const V (*a)[kS], const V (*b)[kS], int i, int j) {
	V t = 0;
#pragma unroll
	for (int rr = 0; rr < kTile; ++rr)
		t = fma(a[rr][i], b[rr][j], t);
	return t;
}

// The last CTA's fold of the per-CTA partials part[b * stride + t] over the
// grid: eight interleaved running sums (eight loads in flight per thread),
// combined in a fixed order -- deterministic for a given grid.
__device__ __forceinline__ double fold_parts(const double *part, int nb, int stride, int t) {
	double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
	for (int b = 0; b < nb; b += 8) {
#pragma unroll
		for (int u = 0; u < 8; ++u)
			if (b + u < nb)
				a[u] += __ldcg(part + (size_t)(b + u) * stride + t);
	}
	return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
}

// Per-CTA partials: one row of kW doubles per CTA (the 16 x 16 Gram entries,
// then up to two 16-value column norms).
constexpr int kW = 256 + 2 * kS;
constexpr int kGroup = 32;  // CTAs per first-level fold group

// Two-level fold of the CTAs' partial rows part[b * kW + t], t < nval: the
// last CTA of each group of kGroup CTAs folds the group's rows (in CTA
// order) into gpart, and the last of those folds the group rows (in group
// order) into res (shared memory).  Returns true in that one CTA.  A fixed
// grouping, so the result is deterministic for a given grid; no CTA waits
// for another.  counters: [0] the groups done, [1 + g] group g's CTAs done.
__device__ bool fold2(const double *part, double *gpart, unsigned *counters, int nval,
                      double *res) {
	__shared__ int s_flag;
	const int G = gridDim.x, g = blockIdx.x / kGroup, ng = (G + kGroup - 1) / kGroup;
	const int b0 = g * kGroup, gsize = min(kGroup, G - b0);
	__threadfence();
	__syncthreads();
	if (threadIdx.x == 0)
		s_flag = atomicAdd(counters + 1 + g, 1u) == (unsigned)(gsize - 1);
	__syncthreads();
	if (!s_flag)
		return false;
	__threadfence();
	for (int t = threadIdx.x; t < nval; t += blockDim.x) {
		double a[4] = {0.0, 0.0, 0.0, 0.0};
		for (int b = 0; b < gsize; b += 4) {
#pragma unroll
			for (int u = 0; u < 4; ++u)
				if (b + u < gsize)
					a[u] += __ldcg(part + (size_t)(b0 + b + u) * kW + t);
		}
		gpart[(size_t)g * kW + t] = (a[0] + a[1]) + (a[2] + a[3]);
	}
	if (threadIdx.x == 0)
		counters[1 + g] = 0;
	__threadfence();
	__syncthreads();
	if (threadIdx.x == 0)
		s_flag = atomicAdd(counters, 1u) == (unsigned)(ng - 1);
	__syncthreads();
	if (!s_flag)
		return false;
	__threadfence();
	for (int t = threadIdx.x; t < nval; t += blockDim.x) {
		double a[4] = {0.0, 0.0, 0.0, 0.0};
		for (int q = 0; q < ng; q += 4) {
#pragma unroll
			for (int u = 0; u < 4; ++u)
				if (q + u < ng)
					a[u] += __ldcg(gpart + (size_t)(q + u) * kW + t);
		}
		res[t] = (a[0] + a[1]) + (a[2] + a[3]);
	}
	if (threadIdx.x == 0)
		counters[0] = 0;
	__syncthreads();
	return true;
}

// X = A^-1 B for the 16 x 16 matrix A with 16 right-hand sides B (both in
// shared memory, row-major, padded rows; B overwritten with the solution):
// Gaussian elimination with partial pivoting by all 256 threads of the CTA.
// Returns false (the same in every thread) on a zero pivot.
struct SmallLs {
	double A[kS][kS + 1], B[kS][kS + 1];
	double fac[kS];
	int piv, ok;
};

__device__ bool small_solve_par(SmallLs &L) {
	const int i = threadIdx.x / kS, j = threadIdx.x % kS;
	if (threadIdx.x == 0)
		L.ok = 1;
	__syncthreads();
	for (int k = 0; k < kS; ++k) {
		if (threadIdx.x < 32) {
			const int lane = threadIdx.x;
			double v = (lane >= k && lane < kS) ? fabs(L.A[lane][k]) : -1.0;
			int idx = lane;
#pragma unroll
			for (int off = 16; off > 0; off >>= 1) {
				const double ov = __shfl_down_sync(0xffffffffu, v, off);
				const int oi = __shfl_down_sync(0xffffffffu, idx, off);
				if (ov > v || (ov == v && oi < idx)) {
					v = ov;
					idx = oi;
				}
			}
			if (lane == 0) {
				L.piv = idx;
				if (!(v > 0.0))
					L.ok = 0;
			}
		}
		__syncthreads();
		if (!L.ok)
			return false;
		const int p = L.piv;
		if (p != k) {
			if (i == 0) {
				const double t = L.A[k][j];
				L.A[k][j] = L.A[p][j];
				L.A[p][j] = t;
			}
			else if (i == 1) {
				const double t = L.B[k][j];
				L.B[k][j] = L.B[p][j];
				L.B[p][j] = t;
			}
		}
		__syncthreads();
		if (threadIdx.x < kS && (int)threadIdx.x > k)
			L.fac[threadIdx.x] = L.A[threadIdx.x][k] / L.A[k][k];
		__syncthreads();
		if (i > k) {
			const double f = L.fac[i];
			if (j >= k)
				L.A[i][j] -= f * L.A[k][j];
			L.B[i][j] -= f * L.B[k][j];
		}
		__syncthreads();
	}
	for (int k = kS - 1; k >= 0; --k) {
		if (threadIdx.x < kS) {
			double s = L.B[k][j];
			for (int m = k + 1; m < kS; ++m)
				s -= L.A[k][m] * L.B[m][j];
			L.B[k][j] = s / L.A[k][k];
		}
		__syncthreads();
	}
	return true;
}

// beta = G^-1 G', G = G' (all threads of the last CTA); false on breakdown
__device__ bool form_beta(BcgState *st, SmallLs &L) {
	const int i = threadIdx.x / kS, j = threadIdx.x % kS;
	L.A[i][j] = st->G[threadIdx.x];
	L.B[i][j] = st->Gn[threadIdx.x];
	__syncthreads();
	const bool ok = small_solve_par(L);
	if (ok)
		st->beta[threadIdx.x] = L.B[i][j];
	st->G[threadIdx.x] = st->Gn[threadIdx.x];
	return ok;
}

// The operator for the block SpMM: a grid stencil in symmetric storage (rows
// addressed by their grid coordinates, every neighbour load independent) or
// the CSR rows.
template<class V>
struct BcgOp {
	const int *rp, *col;
	const V *val;
	const V *S;  // grid: diagonal, upper diagonals (null: CSR)
	int64_t ld;
	int nx, ny, nz, K;
};

// ---------------------------------------------------------------------
// Register-blocked layout of the iteration kernels.  Row phase: a thread
// owns a quad of 4 columns of one row (64 rows per 256-thread step; a warp
// reads 8 rows x 64 contiguous bytes of a block vector with 16-byte loads).
// The 16 x 16 coefficient matrices (alpha, beta) are read 16 bytes at a
// time from shared memory, the step's rows of P / Q / Z / R are staged in
// shared memory (rows padded to kLd values: 16-byte aligned, the 8 rows of a
// warp on distinct banks).  Gram phase: thread (g, a, b) accumulates the 4 x 4
// block [4a, 4a+4) x [4b, 4b+4) of the product over the step rows g, g + 16,
// g + 32, g + 48 (one plain step sum per entry, then a compensated running
// sum); at the end the 16 row groups are folded in a fixed order.
constexpr int kQ = 4;
constexpr int kQRows = 256 / (kS / kQ);  // 64 rows per step
constexpr int kLd = kS + 4;

__device__ __forceinline__ void ld4(const float *p, float (&o)[4]) {
	const float4 t = *reinterpret_cast<const float4 *>(p);
	o[0] = t.x;
	o[1] = t.y;
	o[2] = t.z;
	o[3] = t.w;
}
__device__ __forceinline__ void ld4(const double *p, double (&o)[4]) {
	const double2 t0 = *reinterpret_cast<const double2 *>(p);
	const double2 t1 = *reinterpret_cast<const double2 *>(p + 2);
	o[0] = t0.x;
	o[1] = t0.y;
	o[2] = t1.x;
	o[3] = t1.y;
}
__device__ __forceinline__ void st4(float *p, const float (&o)[4]) {
	*reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
}
__device__ __forceinline__ void st4(double *p, const double (&o)[4]) {
	*reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
	*reinterpret_cast<double2 *>(p + 2) = make_double2(o[2], o[3]);
}
template<class V>
__device__ __forceinline__ void ldg4(const V *p, V (&o)[4]) {
	if constexpr (sizeof(V) == 4) {
		const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
		o[0] = t.x;
		o[1] = t.y;
		o[2] = t.z;
		o[3] = t.w;
	}
	else {
		const double2 t0 = __ldg(reinterpret_cast<const double2 *>(p));
		const double2 t1 = __ldg(reinterpret_cast<const double2 *>(p) + 1);
		o[0] = t0.x;
		o[1] = t0.y;
		o[2] = t1.x;
		o[3] = t1.y;
	}
}

// Gram accumulation of one step: m[a'][b'] += sum over the group's rows of
// za[row][4a + a'] * zb[row][4b + b'] (plain step sums, compensated across
// steps)
template<class V>
struct GramAcc {
	BAcc<V> m[kQ][kQ];
	__device__ void step(const V (*za)[kLd], const V (*zb)[kLd], int g, int a, int b) {
		V t[kQ][kQ];
#pragma unroll
		for (int i = 0; i < kQ; ++i)
#pragma unroll
			for (int j = 0; j < kQ; ++j)
				t[i][j] = 0;
#pragma unroll
		for (int rr = 0; rr < kQRows / 16; ++rr) {
			const int row = g + 16 * rr;
			V u[kQ], w[kQ];
			ld4(&za[row][kQ * a], u);
			ld4(&zb[row][kQ * b], w);
#pragma unroll
			for (int i = 0; i < kQ; ++i)
#pragma unroll
				for (int j = 0; j < kQ; ++j)
					t[i][j] = fma(u[i], w[j], t[i][j]);
		}
#pragma unroll
		for (int i = 0; i < kQ; ++i)
#pragma unroll
			for (int j = 0; j < kQ; ++j)
				m[i][j].add(t[i][j]);
	}
	// the CTA's 16 x 16 sums into part row b (entry i * 16 + j); red holds
	// 8 x 256 doubles of shared memory.  Row groups g and g + 1 share a warp
	// (xor-16 shuffle), the 8 warps' sums are then folded in warp order.
	__device__ void to_part(double *part, double (*red)[256], int g, int a, int b) {
		const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
		__syncthreads();
#pragma unroll
		for (int i = 0; i < kQ; ++i)
#pragma unroll
			for (int j = 0; j < kQ; ++j) {
				double v = m[i][j].get();
				v += __shfl_xor_sync(0xffffffffu, v, 16);
				if (lane < 16)
					red[warp][(kQ * a + i) * kS + kQ * b + j] = v;
			}
		__syncthreads();
		double t = 0.0;
#pragma unroll
		for (int w = 0; w < 8; ++w)
			t += red[w][threadIdx.x];
		part[(size_t)blockIdx.x * kW + threadIdx.x] = t;
	}
};

// q[c] = (A P)[r][4 cq + c], the products in the CSR column order
template<class V>
__device__ __forceinline__ void bcg_row4(const BcgOp<V> &A, const V *__restrict__ P, int r, int cq,
                                         V (&q)[kQ]) {
#pragma unroll
	for (int c = 0; c < kQ; ++c)
		q[c] = 0;
	if (A.S) {
		const int64_t nxy = (int64_t)A.nx * A.ny;
		const int i = r % A.nx;
		const int line = r / A.nx;
		const int jj = A.K >= 2 ? line % A.ny : 0, kk = A.K >= 2 ? line / A.ny : 0;
		const V *U1 = A.S + A.ld, *U2 = A.S + 2 * A.ld, *U3 = A.S + 3 * A.ld;
		const bool has[7] = {A.K >= 3 && kk > 0, A.K >= 2 && jj > 0, i > 0, true,
		                     i < A.nx - 1, A.K >= 2 && jj < A.ny - 1, A.K >= 3 && kk < A.nz - 1};
		const int64_t off[7] = {-nxy, -A.nx, -1, 0, 1, A.nx, nxy};
		// all loads issued before any use: an absent neighbour reads row r
		// itself (an L1 hit) and its products are skipped
		V a[7], x[7][kQ];
#pragma unroll
		for (int t = 0; t < 7; ++t) {
			const V *U = t == 3 ? A.S : (t < 3 ? (t == 0 ? U3 : t == 1 ? U2 : U1)
			                                   : (t == 4 ? U1 : t == 5 ? U2 : U3));
			const int64_t c = has[t] ? r + off[t] : r;
			a[t] = __ldg(U + (t < 3 ? c : r));
			ldg4(P + (size_t)c * kS + kQ * cq, x[t]);
		}
#pragma unroll
		for (int t = 0; t < 7; ++t)
			if (has[t])
#pragma unroll
				for (int c = 0; c < kQ; ++c)
					q[c] = fma(a[t], x[t][c], q[c]);
		return;
	}
	const int k0 = __ldg(A.rp + r), k1 = __ldg(A.rp + r + 1);
	for (int k = k0; k < k1; k += 4) {
		// a batch of up to 4 entries: the column ids, then the gathers
		int col[4];
		V a[4];
#pragma unroll
		for (int t = 0; t < 4; ++t) {
			const int kk = k + t < k1 ? k + t : k1 - 1;
			col[t] = __ldg(A.col + kk);
			a[t] = __ldg(A.val + kk);
		}
		V x[4][kQ];
#pragma unroll
		for (int t = 0; t < 4; ++t)
			ldg4(P + (size_t)col[t] * kS + kQ * cq, x[t]);
#pragma unroll
		for (int t = 0; t < 4; ++t)
			if (k + t < k1)
#pragma unroll
				for (int c = 0; c < kQ; ++c)
					q[c] = fma(a[t], x[t][c], q[c]);
	}
}

// Q = A P and the CTA's part of M = P^T Q; the last CTA forms alpha = M^-1 G
template<class V>
__global__ void __launch_bounds__(256)
k_bcg_spmm(int n, BcgOp<V> A, const V *__restrict__ P, V *__restrict__ Q, BcgState *st,
           double *part, double *gpart, unsigned *counters) {
	__shared__ __align__(16) V sp[kQRows][kLd];
	__shared__ __align__(16) V sq[kQRows][kLd];
	__shared__ double red[8][256];
	__shared__ SmallLs L;
	__shared__ double sres[kW];
	if (bcg_skip(st))
		return;
	const int rs = threadIdx.x >> 2, cq = threadIdx.x & 3;
	const int g = threadIdx.x >> 4, ga = (threadIdx.x >> 2) & 3, gb = threadIdx.x & 3;
	const int nsteps = (n + kQRows - 1) / kQRows;
	GramAcc<V> m;
	for (int t = blockIdx.x; t < nsteps; t += gridDim.x) {
		const int r = t * kQRows + rs;
		V q[kQ], p[kQ];
		if (r < n) {
			bcg_row4(A, P, r, cq, q);
			ldg4(P + (size_t)r * kS + kQ * cq, p);
			st4(Q + (size_t)r * kS + kQ * cq, q);
		}
		else {
#pragma unroll
			for (int c = 0; c < kQ; ++c)
				q[c] = p[c] = 0;
		}
		st4(&sp[rs][kQ * cq], p);
		st4(&sq[rs][kQ * cq], q);
		__syncthreads();
		m.step(sp, sq, g, ga, gb);
		__syncthreads();
	}
	m.to_part(part, red, g, ga, gb);
	if (fold2(part, gpart, counters, 256, sres)) {
		const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
		const double v = sres[threadIdx.x];
		st->M[threadIdx.x] = v;
		L.A[tr][tj] = v;
		L.B[tr][tj] = st->G[threadIdx.x];
		__syncthreads();
		const bool ok = small_solve_par(L);
		if (ok)
			st->alpha[threadIdx.x] = L.B[tr][tj];
		if (threadIdx.x == 0 && !ok) {
			st->done = 1;
			st->status = FS_DIVERGED_BREAKDOWN;
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
             double *gpart, unsigned *counters, double tolf, int maxiter, double delta) {
	__shared__ __align__(16) V sa[kS][kLd];
	__shared__ __align__(16) V sp[kQRows][kLd];
	__shared__ __align__(16) V sq[kQRows][kLd];
	__shared__ double red[8][256];
	__shared__ SmallLs L;
	__shared__ int s_beta;
	__shared__ double sres[kW];
	if (bcg_skip(st))
		return;
	{
		const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
		sa[tr][tj] = (V)st->alpha[threadIdx.x];
	}
	__syncthreads();
	const int rs = threadIdx.x >> 2, cq = threadIdx.x & 3;
	const int g = threadIdx.x >> 4, ga = (threadIdx.x >> 2) & 3, gb = threadIdx.x & 3;
	const int nsteps = (n + kQRows - 1) / kQRows;
	GramAcc<V> gm;
	BAcc<V> nr[kQ];
	for (int t = blockIdx.x; t < nsteps; t += gridDim.x) {
		const int r = t * kQRows + rs;
		V p[kQ], q[kQ], x[kQ], rv[kQ];
		V dr = 0;
		if (r < n) {
			ldg4(P + (size_t)r * kS + kQ * cq, p);
			ldg4(Q + (size_t)r * kS + kQ * cq, q);
			ld4(X + (size_t)r * kS + kQ * cq, x);
			ld4(R + (size_t)r * kS + kQ * cq, rv);
			dr = dinv ? __ldg(dinv + r) : V(1);
		}
		else {
#pragma unroll
			for (int c = 0; c < kQ; ++c)
				p[c] = q[c] = x[c] = rv[c] = 0;
		}
		st4(&sp[rs][kQ * cq], p);
		st4(&sq[rs][kQ * cq], q);
		__syncthreads();
		// x += P[r][:] alpha[:, quad], r -= Q[r][:] alpha[:, quad]
#pragma unroll
		for (int i4 = 0; i4 < kS / kQ; ++i4) {
			V pr[kQ], qr[kQ];
			ld4(&sp[rs][kQ * i4], pr);
			ld4(&sq[rs][kQ * i4], qr);
#pragma unroll
			for (int ii = 0; ii < kQ; ++ii) {
				V al[kQ];
				ld4(&sa[kQ * i4 + ii][kQ * cq], al);
#pragma unroll
				for (int c = 0; c < kQ; ++c) {
					x[c] = fma(pr[ii], al[c], x[c]);
					rv[c] = fma(-qr[ii], al[c], rv[c]);
				}
			}
		}
		V z[kQ];
#pragma unroll
		for (int c = 0; c < kQ; ++c) {
			z[c] = dr * rv[c];
			if (r < n)
				nr[c].add(rv[c] * rv[c]);
		}
		if (r < n) {
			st4(X + (size_t)r * kS + kQ * cq, x);
			st4(R + (size_t)r * kS + kQ * cq, rv);
		}
		else {
#pragma unroll
			for (int c = 0; c < kQ; ++c)
				z[c] = rv[c] = 0;
		}
		__syncthreads();
		// the staged P and Q are consumed: stage Z and R for G' = Z^T R
		st4(&sp[rs][kQ * cq], z);
		st4(&sq[rs][kQ * cq], rv);
		__syncthreads();
		gm.step(sp, sq, g, ga, gb);
		__syncthreads();
	}
	gm.to_part(part, red, g, ga, gb);
	// column norms: this thread's 4 columns, folded over the 64 row slots
	// (in the fold buffer, once every thread has read it)
	double (*cn)[kS] = reinterpret_cast<double (*)[kS]>(&red[0][0]);
	__syncthreads();
#pragma unroll
	for (int c = 0; c < kQ; ++c)
		cn[rs][kQ * cq + c] = nr[c].get();
	__syncthreads();
	if (threadIdx.x < kS) {
		double c = 0.0;
		for (int q = 0; q < kQRows; ++q)
			c += cn[q][threadIdx.x];
		part[(size_t)blockIdx.x * kW + 256 + threadIdx.x] = c;
	}
	if (fold2(part, gpart, counters, 256 + kS, sres)) {
		st->Gn[threadIdx.x] = sres[threadIdx.x];
		if (threadIdx.x < kS)
			st->rnorm[threadIdx.x] = sqrt(sres[256 + threadIdx.x]);
		__syncthreads();
		if (threadIdx.x == 0) {
			const int it = st->iter + 1;
			st->iter = it;
			bool finite = true;
			for (int j = 0; j < kS; ++j)
				finite = finite && isfinite(st->rnorm[j]);
			s_beta = 0;
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
				else
					s_beta = 1;
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
				else
					s_beta = 1;
			}
		}
		__syncthreads();
		if (s_beta && !form_beta(st, L) && threadIdx.x == 0) {
			st->done = 1;
			st->status = FS_DIVERGED_BREAKDOWN;
		}
	}
}

// P = Z + P beta (Z = D^-1 R)
template<class V>
__global__ void __launch_bounds__(256)
k_bcg_dir(int n, V *__restrict__ P, const V *__restrict__ R, const V *__restrict__ dinv,
          const BcgState *st) {
	__shared__ __align__(16) V sb[kS][kLd];
	__shared__ __align__(16) V sp[kQRows][kLd];
	if (bcg_skip(st))
		return;
	{
		const int tr = threadIdx.x / kS, tj = threadIdx.x % kS;
		sb[tr][tj] = (V)st->beta[threadIdx.x];
	}
	const int rs = threadIdx.x >> 2, cq = threadIdx.x & 3;
	const int nsteps = (n + kQRows - 1) / kQRows;
	for (int t = blockIdx.x; t < nsteps; t += gridDim.x) {
		const int r = t * kQRows + rs;
		V p[kQ], pn[kQ];
		if (r < n) {
			ld4(P + (size_t)r * kS + kQ * cq, p);
			ldg4(R + (size_t)r * kS + kQ * cq, pn);
			const V d = dinv ? __ldg(dinv + r) : V(1);
#pragma unroll
			for (int c = 0; c < kQ; ++c)
				pn[c] = d * pn[c];
		}
		else {
#pragma unroll
			for (int c = 0; c < kQ; ++c)
				p[c] = pn[c] = 0;
		}
		__syncthreads();
		st4(&sp[rs][kQ * cq], p);
		__syncthreads();
#pragma unroll
		for (int i4 = 0; i4 < kS / kQ; ++i4) {
			V pr[kQ];
			ld4(&sp[rs][kQ * i4], pr);
#pragma unroll
			for (int ii = 0; ii < kQ; ++ii) {
				V be[kQ];
				ld4(&sb[kQ * i4 + ii][kQ * cq], be);
#pragma unroll
				for (int c = 0; c < kQ; ++c)
					pn[c] = fma(pr[ii], be[c], pn[c]);
			}
		}
		if (r < n)
			st4(P + (size_t)r * kS + kQ * cq, pn);
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
		st->G[threadIdx.x] = fold_parts(part, gridDim.x, 256, threadIdx.x);
		if (threadIdx.x < kS) {
			const double c1 = fold_parts(part2, gridDim.x, 2 * kS, threadIdx.x);
			const double c2 = fold_parts(part2, gridDim.x, 2 * kS, kS + threadIdx.x);
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
	__shared__ SmallLs L;
	__shared__ int s_beta;
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
		st->Gn[threadIdx.x] = fold_parts(part, gridDim.x, 256, threadIdx.x);
		if (threadIdx.x < kS) {
			const double c = fold_parts(part2, gridDim.x, kS, threadIdx.x);
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
			s_beta = 0;
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
			else
				s_beta = 1;
		}
		__syncthreads();
		if (s_beta && !form_beta(st, L) && threadIdx.x == 0) {
			st->done = 1;
			st->status = FS_DIVERGED_BREAKDOWN;
		}
		if (threadIdx.x == 0)
			*counter = 0;
	}
}

struct BcgPlan {
	BcgState *st = nullptr, *hst = nullptr;
	void *work = nullptr;       // P, Q, R (and the FP32 X correction)
	double *part = nullptr;     // per-CTA partial rows (grid x kW) + norm partials
	double *gpart = nullptr;    // per-group partial rows of the two-level fold
	unsigned *counter = nullptr;  // [0] + one per fold group
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
	// every kernel on all SMs at its occupancy (resident CTAs per SM), the
	// partials folded in groups of kGroup CTAs
	const int nsteps = (int)((n + kQRows - 1) / kQRows);
	auto grid_of = [&](auto kern) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, 256, 0) != cudaSuccess || nb < 1)
			nb = 1;
		return std::max(1, std::min(ctx->sms * std::min(nb, 8), nsteps));
	};
	const int G = grid_of(k_bcg_spmm<V>);
	const int Gu = grid_of(k_bcg_update<V>);
	const int Gd = grid_of(k_bcg_dir<V>);
	const size_t m = (size_t)n * kS;
	if (p.n != n) {
		if (p.work) {
			cudaStreamSynchronize(ctx->stream);
			cudaFree(p.work);
			cudaFree(p.part);
			cudaFree(p.gpart);
			cudaFree(p.counter);
			cudaFree(p.st);
			cudaFreeHost(p.hst);
			p = BcgPlan();
		}
		FS_CUDA_TRY(ctx, cudaMalloc(&p.work, sizeof(V) * (mixed ? 4 : 3) * m));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.part, sizeof(double) * (size_t)ctx->sms * 8 * kW));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.gpart,
		                            sizeof(double) * (size_t)(ctx->sms * 8 / kGroup + 2) * kW));
		const size_t cbytes = sizeof(unsigned) * (size_t)(ctx->sms * 8 / kGroup + 2);
		FS_CUDA_TRY(ctx, cudaMalloc(&p.counter, cbytes));
		FS_CUDA_TRY(ctx, cudaMemset(p.counter, 0, cbytes));
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
	// a grid stencil in symmetric storage: neighbours addressed by the grid
	// coordinates; anything else: the CSR rows
	BcgOp<V> op{A->rowptr, A->col, val, nullptr, 0, 0, 0, 0, 0};
	FS_TRY(ensure_sym(A, mixed));
	const int coding = active_coding(A, mixed);
	if (A->grid_nx > 0 && (coding == kCodingSym || coding == kCodingGrid)) {
		op.S = sym_vals<V>(A);
		op.ld = A->sym_ld;
		op.nx = A->grid_nx;
		op.ny = A->grid_ny;
		op.nz = A->grid_nz;
		op.K = A->nsym;
	}
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
			k_bcg_spmm<V><<<G, 256, 0, ctx->stream>>>((int)n, op, Pm, Qm, p.st, part, p.gpart,
			                                          p.counter);
			FS_TRY(check_launch(ctx, "block cg spmm"));
			k_bcg_update<V><<<Gu, 256, 0, ctx->stream>>>((int)n, xv, Pm, R, Qm, dinv, p.st, part,
			                                             p.gpart, p.counter, tolf, maxiter, delta);
			FS_TRY(check_launch(ctx, "block cg update"));
			k_bcg_dir<V><<<Gd, 256, 0, ctx->stream>>>((int)n, Pm, R, dinv, p.st);
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
		return set_err(ctx, FS_ERR_UNSUPPORTED, "block CG: the library takes %d right-hand sides", kS);
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
