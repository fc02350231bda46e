// Device GMRES(m): restarted, left or right preconditioned, with the
// reference's Givens rotations and back-solve (flecsolve/solvers/gmres.hh:
// 78-348).
//
// Orthogonalisation of the new vector v against the basis V_0..V_k:
//  * CGS2 (default): classical Gram-Schmidt applied twice, in three fused
//    passes over V -- (1) h = V^T v; (2) v -= V h and h2 = V^T v in the same
//    pass; (3) v -= V h2 with ||v||^2 -- so a step costs 3 reductions instead
//    of the k + 2 of modified Gram-Schmidt.
//  * MGS: the reference's modified Gram-Schmidt order (gmres.hh:265-279),
//    one fused "v -= h_{j-1} V_{j-1}; h_j = v . V_j" kernel per basis vector.
// The Hessenberg column, the Givens rotations (Bindel, Demmel, Kahan,
// Marques, Algorithm 1), the convergence test and the restart decision run
// in the last block of the final pass, on the device.  One restart cycle
// (m steps + the restart) is one CUDA graph; kernels after a stop return
// immediately.
#include <cmath>
#include <cstring>

#include "solver.cuh"

namespace fsg {

namespace {

constexpr int kT = 256;
constexpr int kChunk = 16;  // basis vectors per orthogonalisation pass
static_assert(kChunk <= kPartPerBlock, "partials buffer holds kPartPerBlock values per CTA");

#define FOR_EACH(i, n)                                                          \
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n);  \
	     i += (int64_t)gridDim.x * blockDim.x)

__device__ __forceinline__ bool stopped(const KState *st) {
	return st->done || (st->flags & KF_RESTART);
}
__device__ __forceinline__ bool restart_pending(const KState *st) {
	return !st->done && (st->flags & KF_RESTART);
}

// ----------------------------------------------- block multi-reduction --

// Sum nv (<= kChunk) per-thread values over the block into part[b*nv + j].
// Fully unrolled over kChunk with a predicate, so the values stay in
// registers (a runtime-bounded loop would move them to local memory).
__device__ __forceinline__ void block_multi_sum(const double (&vals)[kChunk], int nv, double *part,
                                                double *sh) {
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int nw = blockDim.x >> 5;
#pragma unroll
	for (int j = 0; j < kChunk; ++j) {
		if (j < nv) {
			double v = vals[j];
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
				v += __shfl_down_sync(0xffffffffu, v, o);
			if (lane == 0)
				sh[j * 8 + wid] = v;
		}
	}
	__syncthreads();
	if ((int)threadIdx.x < nv) {
		double t = 0.0;
		for (int w = 0; w < nw; ++w)
			t += sh[threadIdx.x * 8 + w];
		part[(size_t)blockIdx.x * nv + threadIdx.x] = t;
	}
}

// Last block: out[j] = sum over blocks of part[b*nv + j].  Every thread sums
// the blocks b = t, t + blockDim, ... (all nv values of a block are adjacent,
// so a warp reads contiguous memory), then the block tree combines the
// threads' sums: a fixed order, so the result is deterministic for a given
// grid, with every thread's loads in flight at once.
__device__ __forceinline__ void fold_multi(const double *part, int nv, double *out, double *sh) {
	double acc[kChunk];
#pragma unroll
	for (int j = 0; j < kChunk; ++j)
		acc[j] = 0.0;
	for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
		for (int j = 0; j < kChunk; ++j)
			if (j < nv)
				acc[j] += __ldcg(part + (size_t)b * nv + j);
	}
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int nw = blockDim.x >> 5;
	__syncthreads();  // sh was used by the block's own reduction
#pragma unroll
	for (int j = 0; j < kChunk; ++j) {
		if (j < nv) {
			double v = acc[j];
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
				v += __shfl_down_sync(0xffffffffu, v, o);
			if (lane == 0)
				sh[j * 8 + wid] = v;
		}
	}
	__syncthreads();
	if ((int)threadIdx.x < nv) {
		double t = 0.0;
		for (int w = 0; w < nw; ++w)
			t += sh[threadIdx.x * 8 + w];
		out[threadIdx.x] = t;
	}
}

// ------------------------------------------- least-squares (device) -----

// gmres.hh:281-296
__device__ void apply_givens(GmState *g, int i, int k) {
	const int ld = g->ld;
	double x = g->H[i + ld * k], y = g->H[i + 1 + ld * k];
	double c = g->cs[i], s = g->sn[i];
	g->H[i + ld * k] = c * x + s * y;
	g->H[i + 1 + ld * k] = -s * x + c * y;
}

// gmres.hh:298-331
__device__ void compute_givens(GmState *g, int k) {
	const int ld = g->ld;
	double f = g->H[k + ld * k], gg = g->H[k + 1 + ld * k];
	double c, s;
	if (gg == 0.0) {
		c = 1.0;
		s = 0.0;
	}
	else if (f == 0.0) {
		c = 0.0;
		s = (gg < 0.0) ? -1.0 : 1.0;
	}
	else {
		double r = sqrt(f * f + gg * gg);
		r = 1.0 / r;
		c = fabs(f) * r;
		s = copysign(gg * r, f);
	}
	g->cs[k] = c;
	g->sn[k] = s;
}

// The Hessenberg column k is in place (H(0..k, k) and H(k+1, k) = vnorm):
// rotations, residual estimate and the stop / restart decision
// (gmres.hh:156-225).  Single thread.
__device__ void finish_step(GmState *g, KState *st, double *hist) {
	const int k = g->k;
	const int ld = g->ld;
	const double vnorm = g->vnorm;
	for (int i = 0; i < k; i++)
		apply_givens(g, i, k);
	if (vnorm != 0.0) {
		compute_givens(g, k);
		apply_givens(g, k, k);
		g->H[k + 1 + ld * k] = 0.0;
		double x = g->dw[k], c = g->cs[k], s = g->sn[k];
		g->dw[k] = c * x;
		g->dw[k + 1] = -s * x;
	}
	const double res = fabs(g->dw[k + 1]);
	g->k = k + 1;
	const int it = st->iter + 1;
	st->iter = it;
	st->res = res;
	if (st->nhist < st->hist_cap)
		hist[st->nhist] = res;
	st->nhist += 1;
	if (!isfinite(res))
		st->flags |= KF_NONFINITE;
	if (res < st->tol) {
		st->done = 1;
		st->status = FS_CONVERGED_RTOL;
		st->info_iters = it;
	}
	else if (it >= st->maxiter || (st->flags & KF_NONFINITE)) {
		st->done = 1;
		st->status = FS_DIVERGED_ITERS;
	}
	else if (g->k == g->m) {
		st->flags |= KF_RESTART;
	}
}

// finish_step by the whole CTA: the column H(0..k+1, k) and the k earlier
// rotations are staged in shared memory (`col`, 3 (k + 2) doubles) by all
// threads, thread 0 runs the same rotations and tests on them, and the
// column is written back by all threads -- the serial chain of global
// loads and stores of the one-thread form costs a few microseconds per
// rotation at large k.  Every thread of the CTA calls it.
__device__ void finish_step_cta(GmState *g, KState *st, double *hist, double *col) {
	const int k = g->k, ld = g->ld, tid = threadIdx.x;
	double *cs = col + (k + 2), *sn = cs + (k + 2);
	for (int i = tid; i <= k + 1; i += blockDim.x)
		col[i] = g->H[i + ld * k];
	for (int i = tid; i < k; i += blockDim.x) {
		cs[i] = g->cs[i];
		sn[i] = g->sn[i];
	}
	__syncthreads();
	if (tid == 0) {
		// the rotations of apply_givens / compute_givens, on the staged column
		for (int i = 0; i < k; i++) {
			const double x = col[i], y = col[i + 1], c = cs[i], s = sn[i];
			col[i] = c * x + s * y;
			col[i + 1] = -s * x + c * y;
		}
		const double vnorm = g->vnorm;
		if (vnorm != 0.0) {
			const double f = col[k], gg = col[k + 1];
			double c, s;
			if (gg == 0.0) {
				c = 1.0;
				s = 0.0;
			}
			else if (f == 0.0) {
				c = 0.0;
				s = (gg < 0.0) ? -1.0 : 1.0;
			}
			else {
				double r = sqrt(f * f + gg * gg);
				r = 1.0 / r;
				c = fabs(f) * r;
				s = copysign(gg * r, f);
			}
			g->cs[k] = c;
			g->sn[k] = s;
			col[k] = c * f + s * gg;
			col[k + 1] = 0.0;
			const double x = g->dw[k];
			g->dw[k] = c * x;
			g->dw[k + 1] = -s * x;
		}
		const double res = fabs(g->dw[k + 1]);
		g->k = k + 1;
		const int it = st->iter + 1;
		st->iter = it;
		st->res = res;
		if (st->nhist < st->hist_cap)
			hist[st->nhist] = res;
		st->nhist += 1;
		if (!isfinite(res))
			st->flags |= KF_NONFINITE;
		if (res < st->tol) {
			st->done = 1;
			st->status = FS_CONVERGED_RTOL;
			st->info_iters = it;
		}
		else if (it >= st->maxiter || (st->flags & KF_NONFINITE)) {
			st->done = 1;
			st->status = FS_DIVERGED_ITERS;
		}
		else if (g->k == g->m) {
			st->flags |= KF_RESTART;
		}
	}
	__syncthreads();
	for (int i = tid; i <= k + 1; i += blockDim.x)
		g->H[i + ld * k] = col[i];
	__syncthreads();
}

// gmres.hh:333-348, nr = k - 1
__device__ void back_solve(GmState *g) {
	const int nr = g->k - 1;
	if (nr < 0)
		return;
	const int ld = g->ld;
	g->dy[nr] = g->dw[nr] / g->H[nr + ld * nr];
	for (int k = nr - 1; k >= 0; k--) {
		g->dy[k] = g->dw[k];
		for (int i = k + 1; i <= nr; i++)
			g->dy[k] -= g->H[k + ld * i] * g->dy[i];
		g->dy[k] = g->dy[k] / g->H[k + ld * k];
	}
}

// ------------------------------------------------------------- kernels --

// v = A z (right: z = D^-1 V_k gathered on the fly) or v = D^-1 A V_k (left)
template<class T>
struct EpiScaleStore {
	static constexpr int NV = 0;
	T *y;
	const T *d;
	const KState *st;
	double *part = nullptr;
	unsigned *counter = nullptr;
	__device__ bool skip() const { return stopped(st); }
	template<class A>
	__device__ void row(int r, T s, A &) const { y[r] = d ? d[r] * s : s; }
	__device__ void finish(const double *) const {}
};

// per-thread partial dot products: FP64 fma for a double basis, FP32 fma
// for a float basis (each thread sums a few dozen terms; the block and grid
// folds are FP64)
__device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }

// Loads of a chunk of basis vectors at element i: all kChunk loads are
// issued before any use (vector indices past `last` repeat `last`, an L1 hit),
// so one element costs one memory round trip, not one per vector.
template<class T>
__device__ __forceinline__ void load_chunk(const T *__restrict__ V, int64_t ld, int j0, int last,
                                           int64_t i, T (&vr)[kChunk]) {
#pragma unroll
	for (int j = 0; j < kChunk; ++j)
		vr[j] = V[(size_t)min(j0 + j, last) * ld + i];
}

// CGS2 pass 1: h1_j = v . V_j, j in [j0, j0 + nj)
template<class T>
__global__ void __launch_bounds__(kT)
k_gm_dots(int64_t n, const T *__restrict__ V, int64_t ld, int j0, int nj,
          const T *__restrict__ v, GmState *g, KState *st, double *part, unsigned *counter) {
	__shared__ double sh[kChunk * 8];
	if (stopped(st))
		return;
	T acc[kChunk];
#pragma unroll
	for (int j = 0; j < kChunk; ++j)
		acc[j] = T(0);
	FOR_EACH(i, n) {
		T vr[kChunk];
		load_chunk(V, ld, j0, j0 + nj - 1, i, vr);
		const T vi = v[i];
#pragma unroll
		for (int j = 0; j < kChunk; ++j)
			if (j < nj)
				acc[j] = mad(vi, vr[j], acc[j]);
	}
	double accd[kChunk];
#pragma unroll
	for (int j = 0; j < kChunk; ++j)
		accd[j] = (double)acc[j];
	block_multi_sum(accd, nj, part, sh);
	if (last_block(counter)) {
		fold_multi(part, nj, g->h1 + j0, sh);
		if (threadIdx.x == 0)
			*counter = 0;
	}
}

// CGS2 pass 2: (chunk j0 == 0 only) v -= sum_j h1_j V_j over all k + 1
// vectors, then h2_j = v . V_j for the chunk [j0, j0 + nj).  The update
// walks the basis a chunk at a time (each chunk's loads issued together); the
// first chunk's vectors stay in registers for the dots of chunk 0.
template<class T>
__global__ void __launch_bounds__(kT)
k_gm_project_dots(int64_t n, const T *__restrict__ V, int64_t ld, int kp1, int j0, int nj,
                  T *__restrict__ v, GmState *g, KState *st, double *part,
                  unsigned *counter) {
	__shared__ double sh[kChunk * 8];
	__shared__ T hs[kGmMaxDim + 1];
	if (stopped(st))
		return;
	for (int j = threadIdx.x; j < kp1; j += blockDim.x)
		hs[j] = (T)g->h1[j];
	__syncthreads();
	T acc[kChunk];
#pragma unroll
	for (int j = 0; j < kChunk; ++j)
		acc[j] = T(0);
	FOR_EACH(i, n) {
		T vr[kChunk];
		T vi = v[i];
		if (j0 == 0) {
			for (int c0 = 0; c0 < kp1; c0 += kChunk) {
				T vc[kChunk];
				load_chunk(V, ld, c0, kp1 - 1, i, vc);
#pragma unroll
				for (int j = 0; j < kChunk; ++j) {
					if (c0 + j < kp1)
						vi = mad(-hs[c0 + j], vc[j], vi);
					if (c0 == 0)
						vr[j] = vc[j];
				}
			}
			v[i] = vi;
		}
		else
			load_chunk(V, ld, j0, j0 + nj - 1, i, vr);
#pragma unroll
		for (int j = 0; j < kChunk; ++j)
			if (j < nj)
				acc[j] = mad(vi, vr[j], acc[j]);
	}
	double accd[kChunk];
#pragma unroll
	for (int j = 0; j < kChunk; ++j)
		accd[j] = (double)acc[j];
	block_multi_sum(accd, nj, part, sh);
	if (last_block(counter)) {
		fold_multi(part, nj, g->h2 + j0, sh);
		if (threadIdx.x == 0)
			*counter = 0;
	}
}

// CGS2 pass 3: v -= sum_j h2_j V_j and ||v||^2; the last block assembles the
// Hessenberg column (h1 + h2, ||v||) and finishes the step
template<class T>
__global__ void __launch_bounds__(kT)
k_gm_project_norm(int64_t n, const T *__restrict__ V, int64_t ld, int kp1,
                  T *__restrict__ v, GmState *g, KState *st, double *part,
                  unsigned *counter, double *hist) {
	__shared__ double sh[128];
	__shared__ T hs[kGmMaxDim + 1];
	if (stopped(st))
		return;
	for (int j = threadIdx.x; j < kp1; j += blockDim.x)
		hs[j] = (T)g->h2[j];
	__syncthreads();
	T acc = T(0);
	FOR_EACH(i, n) {
		T vi = v[i];
		for (int c0 = 0; c0 < kp1; c0 += kChunk) {
			T vc[kChunk];
			load_chunk(V, ld, c0, kp1 - 1, i, vc);
#pragma unroll
			for (int j = 0; j < kChunk; ++j)
				if (c0 + j < kp1)
					vi = mad(-hs[c0 + j], vc[j], vi);
		}
		v[i] = vi;
		acc = mad(vi, vi, acc);
	}
	double accd[1] = {(double)acc};
	block_sum<1>(accd, sh);
	if (threadIdx.x == 0)
		part[blockIdx.x] = accd[0];
	if (last_block(counter)) {
		double s[1];
		sum_partials<1>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			const int k = g->k, ldh = g->ld;
			for (int j = 0; j < kp1; ++j)
				g->H[j + ldh * k] = g->h1[j] + g->h2[j];
			const double vn = sqrt(s[0]);
			g->H[k + 1 + ldh * k] = vn;
			g->vnorm = vn;
			finish_step(g, st, hist);
			*counter = 0;
		}
	}
}

// MGS pass j (gmres.hh:270-278): v -= h_{j-1} V_{j-1} (j > 0), then
// h_j = v . V_j into H(j, k); pass j == kp1 applies the last update, takes
// ||v|| and finishes the step
template<class T>
__global__ void __launch_bounds__(kT)
k_gm_mgs(int64_t n, const T *__restrict__ V, int64_t ld, int j, int kp1,
         T *__restrict__ v, GmState *g, KState *st, double *part, unsigned *counter,
         double *hist) {
	__shared__ double sh[128];
	if (stopped(st))
		return;
	const int k = g->k, ldh = g->ld;
	const T hprev = j > 0 ? (T)g->H[(j - 1) + ldh * k] : T(0);
	const T *Vp = j > 0 ? V + (size_t)(j - 1) * ld : nullptr;
	const T *Vj = j < kp1 ? V + (size_t)j * ld : nullptr;
	T acc = T(0);
	FOR_EACH(i, n) {
		T vi = v[i];
		if (j > 0) {
			vi = mad(-hprev, Vp[i], vi);
			v[i] = vi;
		}
		acc = mad(vi, j < kp1 ? Vj[i] : vi, acc);
	}
	double accd[1] = {(double)acc};
	block_sum<1>(accd, sh);
	if (threadIdx.x == 0)
		part[blockIdx.x] = accd[0];
	if (last_block(counter)) {
		double s[1];
		sum_partials<1>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			if (j < kp1) {
				g->H[j + ldh * k] = s[0];
			}
			else {
				const double vn = sqrt(s[0]);
				g->H[kp1 + ldh * k] = vn;
				g->vnorm = vn;
				finish_step(g, st, hist);
			}
			*counter = 0;
		}
	}
}

// basis_{k+1} = v * (1 / vnorm), or v itself when vnorm == 0
// (gmres.hh:156-162); unused (and skipped) once the step stopped or restarts
template<class T>
__global__ void k_gm_normalize(int64_t n, const T *__restrict__ v, T *__restrict__ out,
                               const GmState *g, const KState *st) {
	if (stopped(st))
		return;
	const double vn = g->vnorm;
	const T inv = (T)(vn != 0.0 ? 1.0 / vn : 1.0);
	FOR_EACH(i, n) out[i] = vn != 0.0 ? v[i] * inv : v[i];
}

// back-solve: GATED = only when a restart is pending
template<bool GATED>
__global__ void k_gm_backsolve(GmState *g, const KState *st) {
	if (GATED && !restart_pending(st))
		return;
	back_solve(g);
}

// correct (gmres.hh:244-263) with nr = k - 1: right: z = sum_i dy_i V_i
// accumulated left to right, x += 1.0 * P z; left: x += dy_i V_i in order.
// x and the accumulation are FP64 for either basis type.
template<bool GATED, class T>
__global__ void __launch_bounds__(kT)
k_gm_correct(int64_t n, const T *__restrict__ V, int64_t ld, const GmState *g,
             const double *__restrict__ dinv, double *__restrict__ x, int right, const KState *st) {
	if (GATED && !restart_pending(st))
		return;
	const int nr = g->k - 1;
	if (nr < 0)
		return;
	__shared__ double dy[kGmMaxDim + 1];
	for (int j = threadIdx.x; j <= nr; j += blockDim.x)
		dy[j] = g->dy[j];
	__syncthreads();
	FOR_EACH(i, n) {
		if (right) {
			double z = 0.0;
			for (int j = 0; j <= nr; ++j)
				z = fma(dy[j], (double)V[(size_t)j * ld + i], z);
			const double pz = dinv ? dinv[i] * z : z;
			x[i] = fma(1.0, pz, x[i]);
		}
		else {
			double xi = x[i];
			for (int j = 0; j <= nr; ++j)
				xi = fma(dy[j], (double)V[(size_t)j * ld + i], xi);
			x[i] = xi;
		}
	}
}

// residual for a (re)start: res = b - A x (right) or D^-1 (b - A x) (left)
// and ||res|| -> st->aux[2]; gated variant runs only with a restart pending
struct EpiGmResidual {
	static constexpr int NV = 1;
	const double *b;
	double *res;
	const double *dleft;
	KState *st;
	double *part;
	unsigned *counter;
	bool gated;
	__device__ bool skip() const { return gated && !restart_pending(st); }
	template<class A>
	__device__ void row(int r, double s, A &acc) const {
		double v = b[r] - s;
		if (dleft)
			v = dleft[r] * v;
		res[r] = v;
		acc.add_prod(0, v, v);
	}
	__device__ void finish(const double *s) const { st->aux[2] = sqrt(s[0]); }
};

// basis_0 = res * (1 / beta), dw[0] = beta, k = 0 (gmres.hh:134-139,
// 218-224); the restart variant also counts the restart and clears the flag
template<bool RESTART, class T>
__global__ void __launch_bounds__(kT)
k_gm_basis0(int64_t n, const double *__restrict__ res, T *__restrict__ V0, GmState *g,
            KState *st, unsigned *counter) {
	if (RESTART && !restart_pending(st))
		return;
	const double beta = st->aux[2];
	const double inv = 1.0 / beta;
	FOR_EACH(i, n) V0[i] = (T)(res[i] * inv);
	if (last_block(counter) && threadIdx.x == 0) {
		g->dw[0] = beta;
		g->k = 0;
		if (RESTART) {
			st->restarts += 1;
			st->flags &= ~KF_RESTART;
		}
		*counter = 0;
	}
}

// start-of-solve test (gmres.hh:125-132) and the Hessenberg geometry
__global__ void k_gm_start(GmState *g, KState *st, int m, int ld) {
	const double beta = st->aux[2];
	st->res0 = beta;
	st->res = beta;
	g->k = 0;
	g->m = m;
	g->ld = ld;
	if (beta < st->tol) {
		st->done = 1;
		st->status = FS_CONVERGED_RTOL;
	}
	else if (st->maxiter <= 0) {
		st->done = 1;
		st->status = FS_DIVERGED_ITERS;
	}
}

// Mixed precision: a cycle ends on the Arnoldi estimate (converged, maxiter
// or k == m); the stopping decision is then taken on the FP64 true residual
// that the restart tail computed into aux[2].
__global__ void k_gm_mixed_decide(KState *st) {
	if (st->done)
		return;
	const double beta = st->aux[2];
	st->res = beta;
	if (!isfinite(beta))
		st->flags |= KF_NONFINITE;
	if (beta < st->tol) {
		st->done = 1;
		st->status = FS_CONVERGED_RTOL;
		st->info_iters = st->iter;
	}
	else if (st->iter >= st->maxiter || (st->flags & KF_NONFINITE)) {
		st->done = 1;
		st->status = FS_DIVERGED_ITERS;
	}
}

// In mixed mode the step's stop tests become "end the cycle"
__global__ void k_gm_mixed_cycle_end(KState *st) {
	if (st->done && st->status == FS_CONVERGED_RTOL) {
		// the FP32 Arnoldi estimate met the tolerance: verify in FP64
		st->done = 0;
		st->status = FS_STATUS_UNKNOWN;
		st->info_iters = 0;
		st->flags |= KF_RESTART;
	}
	else if (st->done && st->status == FS_DIVERGED_ITERS && !(st->flags & KF_NONFINITE)) {
		// maxiter: still fold the cycle into x and measure the residual
		st->done = 0;
		st->flags |= KF_RESTART;
	}
}

}  // namespace
}  // namespace fsg

#include "gmres_staged.cuh"

namespace fsg {

// ---------------------------------------------------------------- host --

namespace {

template<class T>
struct GmBufs {
	T *V;           // basis, ld x (mdim + 1)
	T *v;           // new direction
	const T *dinv;  // Jacobi diagonal in T (or null)
	const T *vals;  // CSR values in T
};

struct GmArgs {
	Vec *b, *x;
	int first, last;   // steps captured
	bool with_restart; // the gated restart tail
	bool mixed;
};

inline GmState *gm_state(Solver *s) { return reinterpret_cast<GmState *>(s->hdev); }
inline int64_t gm_ld(const Solver *s) { return (s->n + 31) / 32 * 32; }

template<class T>
GmBufs<T> gm_bufs(Solver *s) {
	if constexpr (sizeof(T) == 8)
		return {(T *)s->basis, (T *)s->w64[2], (const T *)s->dinv64(), (const T *)s->A->val};
	else
		return {(T *)s->basis, (T *)s->w32[2], (const T *)s->dinv32(), (const T *)s->A->val32};
}

template<class T>
int gm_step(Solver *s, int k) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n, ld = gm_ld(s);
	const int G = red_grid(ctx, n);
	const bool right = s->set.pre_side != FS_LEFT;
	GmBufs<T> B = gm_bufs<T>(s);
	GmState *g = gm_state(s);
	const int kp1 = k + 1;
	const T *Vk = B.V + (size_t)k * ld;
	if (right && B.dinv)
		FS_TRY((launch_spmv<T, false, true>(ctx, s->A, B.vals, Vk, B.dinv,
		                                    EpiScaleStore<T>{B.v, nullptr, s->st})));
	else
		FS_TRY((launch_spmv<T, false, false>(ctx, s->A, B.vals, Vk, nullptr,
		                                     EpiScaleStore<T>{B.v, right ? nullptr : B.dinv, s->st})));
	const bool mgs = !s->gm_delayed && (s->set.ortho == FS_ORTHO_MGS ||
	                                    (s->set.ortho == FS_ORTHO_AUTO && sizeof(T) == 8));
	if (mgs) {
		for (int j = 0; j <= kp1; ++j) {
			k_gm_mgs<T><<<G, kT, 0, ctx->stream>>>(n, B.V, ld, j, kp1, B.v, g, s->st, s->part,
			                                       s->counter, s->hist);
			FS_TRY(check_launch(ctx, "gmres mgs"));
		}
	}
	else if (s->gm_delayed) {
		// delayed CGS2: column k holds u_k; pass 4 finishes column k - 1 and
		// pass 5 writes q_k over u_k and u_{k+1} into column k + 1
		OrthoArgs<T> oa{B.v, B.V + (size_t)kp1 * ld, B.V + (size_t)k * ld, n, kp1,
		                staged_stages(kp1), staged_stride(kp1), g, s->st, s->part, s->counter,
		                s->hist, ctx->dev_err};
		const BasisMaps &map = *reinterpret_cast<const BasisMaps *>(s->gm_map);
		FS_TRY((staged_pass<T, 4>(ctx, oa, map)));
		return staged_pass<T, 5>(ctx, oa, map);
	}
	else if (kp1 <= kStagedMax && s->gm_map_base == (const void *)B.V) {
		// staged CGS2: three passes, the last one writes V_{k+1}
		OrthoArgs<T> oa{B.v, B.V + (size_t)kp1 * ld, nullptr, n, kp1, staged_stages(kp1),
		                staged_stride(kp1), g, s->st, s->part, s->counter, s->hist, ctx->dev_err};
		const BasisMaps &map = *reinterpret_cast<const BasisMaps *>(s->gm_map);
		FS_TRY((staged_pass<T, 1>(ctx, oa, map)));
		FS_TRY((staged_pass<T, 2>(ctx, oa, map)));
		return staged_pass<T, 3>(ctx, oa, map);
	}
	else {
		for (int j0 = 0; j0 < kp1; j0 += kChunk) {
			k_gm_dots<T><<<G, kT, 0, ctx->stream>>>(n, B.V, ld, j0, std::min(kChunk, kp1 - j0), B.v,
			                                        g, s->st, s->part, s->counter);
			FS_TRY(check_launch(ctx, "gmres dots"));
		}
		for (int j0 = 0; j0 < kp1; j0 += kChunk) {
			k_gm_project_dots<T><<<G, kT, 0, ctx->stream>>>(n, B.V, ld, kp1, j0,
			                                                std::min(kChunk, kp1 - j0), B.v, g,
			                                                s->st, s->part, s->counter);
			FS_TRY(check_launch(ctx, "gmres project"));
		}
		k_gm_project_norm<T><<<G, kT, 0, ctx->stream>>>(n, B.V, ld, kp1, B.v, g, s->st, s->part,
		                                                s->counter, s->hist);
		FS_TRY(check_launch(ctx, "gmres norm"));
	}
	k_gm_normalize<T><<<G, kT, 0, ctx->stream>>>(n, B.v, B.V + (size_t)kp1 * ld, g, s->st);
	return check_launch(ctx, "gmres normalize");
}

// residual (FP64) + basis_0 (initial: unconditional; restart: gated)
template<bool RESTART, class T>
int gm_restart(Solver *s, Vec *b, Vec *x) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const bool right = s->set.pre_side != FS_LEFT;
	double *res = s->w64[0];
	FS_TRY((launch_spmv<double, false, false>(
		ctx, s->A, s->A->val, (const double *)x->d, nullptr,
		EpiGmResidual{(const double *)b->d, res, right ? nullptr : s->dinv64(), s->st, s->part,
		              s->counter, RESTART})));
	k_gm_basis0<RESTART, T><<<red_grid(ctx, n), kT, 0, ctx->stream>>>(n, res, (T *)s->basis,
	                                                                 gm_state(s), s->st, s->counter);
	return check_launch(ctx, "gmres basis0");
}

template<class T>
int gm_body(Solver *s, void *a) {
	GmArgs *ga = (GmArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	for (int j = ga->first; j <= ga->last; ++j)
		FS_TRY(gm_step<T>(s, j));
	if (ga->with_restart && s->gm_delayed) {
		// delayed CGS2: the cycle's last column is finished from u_m
		// (column m = last + 1) by one more pass of dots
		const int kp1 = ga->last + 2;
		const int64_t ld = gm_ld(s);
		T *V = (T *)s->basis;
		OrthoArgs<T> oa{V + (size_t)(kp1 - 1) * ld, nullptr, nullptr, n, kp1, staged_stages(kp1),
		                staged_stride(kp1), gm_state(s), s->st, s->part, s->counter, s->hist,
		                ctx->dev_err};
		FS_TRY((staged_pass<T, 6>(ctx, oa, *reinterpret_cast<const BasisMaps *>(s->gm_map))));
	}
	if (ga->with_restart) {
		const bool right = s->set.pre_side != FS_LEFT;
		if (ga->mixed) {
			k_gm_mixed_cycle_end<<<1, 1, 0, ctx->stream>>>(s->st);
			FS_TRY(check_launch(ctx, "gmres cycle end"));
		}
		k_gm_backsolve<true><<<1, 1, 0, ctx->stream>>>(gm_state(s), s->st);
		FS_TRY(check_launch(ctx, "gmres backsolve"));
		k_gm_correct<true, T><<<red_grid(ctx, n), kT, 0, ctx->stream>>>(
			n, (const T *)s->basis, gm_ld(s), gm_state(s), s->dinv64(), (double *)ga->x->d,
			right ? 1 : 0, s->st);
		FS_TRY(check_launch(ctx, "gmres correct"));
		if (ga->mixed) {
			// the true FP64 residual re-anchors the next FP32 cycle
			FS_TRY((launch_spmv<double, false, false>(
				ctx, s->A, s->A->val, (const double *)ga->x->d, nullptr,
				EpiGmResidual{(const double *)ga->b->d, s->w64[0], right ? nullptr : s->dinv64(),
				              s->st, s->part, s->counter, true})));
			k_gm_mixed_decide<<<1, 1, 0, ctx->stream>>>(s->st);
			FS_TRY(check_launch(ctx, "gmres decide"));
			k_gm_basis0<true, T><<<red_grid(ctx, n), kT, 0, ctx->stream>>>(
				n, s->w64[0], (T *)s->basis, gm_state(s), s->st, s->counter);
			FS_TRY(check_launch(ctx, "gmres basis0"));
		}
		else {
			FS_TRY((gm_restart<true, T>(s, ga->b, ga->x)));
		}
	}
	return FS_OK;
}

template<class T>
int gmres_run(Solver *s, Vec *b, Vec *x, fs_solve_info *info, bool mixed) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n, ld = gm_ld(s);
	const bool zg = s->set.base.use_zero_guess != 0;
	const bool right = s->set.pre_side != FS_LEFT;
	const int maxiter = s->set.base.maxiter;
	const int m = s->set.max_krylov_dim < 0 ? maxiter : s->set.max_krylov_dim;
	if (m > kGmMaxDim || (!s->set.restart && maxiter > m))
		return set_err(ctx, FS_ERR_BREAKDOWN,
		               "GMRES settings fail the reference's validate() (gmres.hh:394-404)");
	const int mdim = std::max(1, std::min(m, maxiter));  // gmres.hh:58
	const int cols = mdim + 1;
	const size_t need = sizeof(T) * (size_t)ld * cols;
	if (s->basis_bytes < need) {
		if (s->basis)
			cudaFree(s->basis);
		s->basis = nullptr;
		FS_CUDA_TRY(ctx, cudaMalloc(&s->basis, need));
		FS_CUDA_TRY(ctx, cudaMemsetAsync(s->basis, 0, need, ctx->stream));
		s->basis_bytes = need;
		// graphs captured with the old basis address are stale
		for (auto &kv : s->graphs)
			cudaGraphExecDestroy(kv.second.exec);
		s->graphs.clear();
	}
	{
		// the staged CGS2 passes read the basis through a tensor map (encoded
		// on the host, once per basis, type and shape); without one the
		// register passes run
		const int key[3] = {(int)sizeof(T), cols, (int)(n & 0x7fffffff)};
		if (s->gm_map_base != s->basis || memcmp(key, s->gm_map_key, sizeof key) != 0) {
			s->gm_map_base = nullptr;
			static_assert(sizeof(BasisMaps) <= sizeof(s->gm_map), "tensor map storage");
			if (encode_basis_maps<T>(reinterpret_cast<BasisMaps *>(s->gm_map), (const T *)s->basis,
			                         n, ld, cols)) {
				s->gm_map_base = s->basis;
				memcpy(s->gm_map_key, key, sizeof key);
			}
		}
	}
	// the delayed CGS2 needs the staged passes for every column of a cycle,
	// including the last pass over m + 1 columns; with a diagnostic on the
	// FP64 path (one graph a step, the restart tail in the last step's graph)
	// CGS2 runs, so that a stop by the diagnostic leaves x at that step
	const bool want_delayed =
		s->set.ortho == FS_ORTHO_DCGS2 || (s->set.ortho == FS_ORTHO_AUTO && sizeof(T) == 4);
	s->gm_delayed = want_delayed && s->gm_map_base == s->basis && cols <= kStagedMax &&
	                (mixed || !s->diag);
	FS_CUDA_TRY(ctx, cudaMemsetAsync(s->hdev, 0, sizeof(GmState), ctx->stream));
	FS_TRY(solver_hist(s, std::max(1, maxiter)));
	{
		KState h{};
		h.rtol = (double)s->set.base.rtol;
		h.maxiter = maxiter;
		h.status = FS_STATUS_UNKNOWN;
		h.hist_cap = s->hist_cap;
		FS_CUDA_TRY(ctx, cudaMemcpyAsync(s->st, &h, sizeof(KState), cudaMemcpyHostToDevice, ctx->stream));
		FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	}
	FS_TRY(solver_norms(s, b, x, !zg, 1));
	if (zg)
		FS_CUDA_TRY(ctx, cudaMemsetAsync(x->d, 0, x->bytes(), ctx->stream));
	// initial residual (a zero guess makes b - A x == b exactly, the copy of
	// gmres.hh:112-120), basis_0 and the start test
	FS_TRY((gm_restart<false, T>(s, b, x)));
	GmState *g = gm_state(s);
	k_gm_start<<<1, 1, 0, ctx->stream>>>(g, s->st, m, mdim + 1);
	FS_TRY(check_launch(ctx, "gmres start"));
	FS_TRY(read_state(s));
	const int steps = std::min(m, maxiter);
	const int tag = (mixed ? 1 : 0) + 2 * (int)sizeof(T) + (s->gm_delayed ? 20 : 0);
	int user_stop = 0;
	int64_t seen = 0;
	while (!s->hst->done && !user_stop) {
		if (s->diag && !mixed) {
			// one graph per step so that the diagnostic sees every iteration
			// (x is constant within a cycle, as in the reference)
			for (int j = 0; j < steps && !s->hst->done; ++j) {
				GmArgs a{b, x, j, j, j == steps - 1, mixed};
				FS_TRY(graph_run(s, GraphKey{b->d, x->d, 300000 + 2 * j + (j == steps - 1) + 1000 * tag},
				                 gm_body<T>, &a));
				FS_TRY(read_state(s));
				// one call per new estimate
				const int64_t upto = std::min<int64_t>(s->hst->nhist, s->hist_cap);
				if (upto > seen) {
					double hv[2] = {0, 0};
					const int64_t cnt = std::min<int64_t>(upto - seen, 2);
					FS_CUDA_TRY(ctx, cudaMemcpy(hv, s->hist + (upto - cnt), cnt * sizeof(double),
					                            cudaMemcpyDeviceToHost));
					for (int64_t e = 0; e < cnt && !user_stop; ++e)
						if (s->diag(s->diag_user, reinterpret_cast<fs_vec>(x), hv[e]))
							user_stop = (int)(upto - cnt + e + 1);
					seen = upto;
					if (user_stop)
						break;
				}
			}
		}
		else {
			GmArgs a{b, x, 0, steps - 1, true, mixed};
			FS_TRY(graph_run(s, GraphKey{b->d, x->d, 200000 + steps + 1000 * tag}, gm_body<T>, &a));
			FS_TRY(read_state(s));
			if (s->diag && s->hst->nhist > seen) {
				// mixed: the diagnostic sees each step's estimate after its cycle
				const int64_t upto = std::min<int64_t>(s->hst->nhist, s->hist_cap);
				std::vector<double> hh(upto > seen ? upto - seen : 0);
				if (!hh.empty())
					FS_CUDA_TRY(ctx, cudaMemcpy(hh.data(), s->hist + seen, hh.size() * sizeof(double),
					                            cudaMemcpyDeviceToHost));
				for (size_t j = 0; j < hh.size() && !user_stop; ++j)
					if (s->diag(s->diag_user, reinterpret_cast<fs_vec>(x), hh[j]))
						user_stop = (int)(seen + j + 1);
				seen = upto;
			}
		}
	}
	const int G = red_grid(ctx, n);
	if (!mixed || user_stop) {
		// final correction with the current k (gmres.hh:228-233); in mixed
		// mode every cycle was already folded into x by its tail
		k_gm_backsolve<false><<<1, 1, 0, ctx->stream>>>(g, s->st);
		FS_TRY(check_launch(ctx, "gmres backsolve"));
		k_gm_correct<false, T><<<G, kT, 0, ctx->stream>>>(n, (const T *)s->basis, ld, g, s->dinv64(),
		                                                  (double *)x->d, right ? 1 : 0, s->st);
		FS_TRY(check_launch(ctx, "gmres correct"));
	}
	FS_TRY(read_state(s));
	KState &h = *s->hst;
	s->hhist_count = std::min<int64_t>(h.nhist, s->hist_cap);
	s->mixed_outer = mixed ? h.restarts : 0;
	s->mixed_inner = mixed ? h.iter : 0;
	double xn = 0;
	FS_TRY(fs_vec_l2norm(reinterpret_cast<fs_vec>(x), &xn));
	memset(info, 0, sizeof(*info));
	info->rhs_norm = (float)h.rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)h.sol0;
	info->res_norm_initial = (float)h.res0;
	info->res_norm_final = (float)h.res;
	info->sol_norm_final = (float)xn;
	info->restarts = h.restarts;
	if (user_stop) {
		info->status = FS_CONVERGED_USER;
		info->iters = user_stop;
	}
	else {
		info->status = h.status;
		info->iters = h.info_iters;
		if (h.res0 >= h.tol && info->iters == 0)
			info->status = FS_DIVERGED_ITERS;  // gmres.hh:237-238
	}
	if (h.flags & KF_NONFINITE)
		return set_err(ctx, FS_ERR_NON_FINITE, "GMRES: non-finite residual norm");
	return FS_OK;
}

}  // namespace

int gmres_apply(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	return gmres_run<double>(s, b, x, info, false);
}

int gmres_apply_mixed(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	return gmres_run<float>(s, b, x, info, true);
}

}  // namespace fsg
