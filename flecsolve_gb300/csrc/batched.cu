// Batched solves: many independent systems of uneven size in one persistent
// launch.
//
// The systems are the diagonal blocks of one block-diagonal CSR matrix
// (rows [off[s], off[s+1]) couple only among themselves).  A team owns one
// system and runs its whole Jacobi-PCG loop without leaving the kernel:
//  * the `nbig` largest systems each get a whole thread-block cluster: each
//    CTA owns a contiguous slice of the system's rows, the per-iteration
//    reductions are folded through distributed shared memory (every CTA
//    reads the cluster's partials in rank order, so all CTAs obtain the same
//    bits), and hardware cluster barriers order the phases;
//  * every other system gets one CTA of a cluster (the cluster's CTAs run
//    independent systems; block reductions and block barriers only).
// The split keeps the largest systems -- the batch's critical path: the most
// rows and the most iterations -- from running on one SM while the small
// ones finish elsewhere.
// A system stops on its own convergence test; the rest of the grid keeps
// working (per-system convergence masks without any host round trip).
//
// Arithmetic (the reference's cg.hh:43-139 recurrences): FP64 iterations
// until the residual is below `head` ||b|| (the first decades, where the
// solution's large components form; FP32 recurrences from the first
// iteration lose orthogonality on the larger 2-D systems and take up to 13 %
// more iterations), then FP32 values and vectors, the dots' FP32 products
// summed in compensated FP32 pairs per thread and in FP64 across the team;
// the residual is replaced by the FP64 one, b - A x with the FP64 values,
// whenever it has dropped by `delta` and at every stop, and the stopping test
// is on that FP64 residual.
//
// Storage: a batch whose systems are all symmetric 5-point stencils on square
// grids reads their diagonals and upper diagonals (no column ids; the CSR
// row loop's bits), other batches the CSR.  The row loops take one row at a
// time in the 1024-thread build and 4 or 8 FP32 rows (2 or 4 FP64) in the
// 512- and 256-thread builds, every load of a batch of rows issued before
// any store.
//
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>
#include <vector>

#include "solver.cuh"

namespace cgrp = cooperative_groups;

namespace fsg {

namespace {

struct BatchArgs {
	int nsys;
	int nbig;                // systems 0..nbig-1 of `order` own a whole cluster
	const int *order;        // system processed by cluster c (largest first)
	const int64_t *off;      // row offsets, nsys + 1
	const int *rowptr;
	const int *col;
	const float *val32;
	const double *val64;
	const float *dinv32;
	const double *dinv64;
	const double *b;
	double *x;               // FP64 solution
	float *x32, *r32, *p32, *w32;  // FP32 work (correction, residual, direction, A p)
	double *r64, *p64, *w64;       // FP64 work of the head phase
	fs_solve_info *info;     // per system
	int maxiter;
	float rtol;
	double delta;
	double head;             // FP64 iterations until ||r|| < head ||b|| (0: none)
	int zero_guess;
	// 2-D grid stencils (every system a 5-point operator on an s x s grid
	// with symmetric values, found when the plan is made): the diagonal and
	// the two upper diagonals a(r, r+1), a(r, r+s), FP64 and FP32, and each
	// system's side; null when the batch is not all grid stencils
	const int *side;
	const double *gd64, *gu1_64, *gu2_64;
	const float *gd32, *gu1_32, *gu2_32;
};

__device__ __forceinline__ float fmav(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmav(double a, double b, double c) { return fma(a, b, c); }

// Rows r0 + tid, r0 + tid + nt, ... of one system, U at a time: `load`
// reads every value a row needs into registers for all U rows before `store`
// writes any of them, so each thread keeps U rows' loads in flight at once
// (the compiler cannot move a load above a store that it cannot prove
// disjoint).  The loads are unconditional -- a row past r1 loads row r1 - 1
// again and is not stored -- so that no branch separates them.
template<int U, class L, class S>
__device__ __forceinline__ void rows_batched(int64_t r0, int64_t r1, int tid, int nt, L &&load,
                                             S &&store) {
	using T = decltype(load(r0));
	for (int64_t i0 = r0 + tid; i0 < r1; i0 += (int64_t)U * nt) {
		T t[U];
#pragma unroll
		for (int u = 0; u < U; ++u) {
			const int64_t i = i0 + (int64_t)u * nt;
			t[u] = load(i < r1 ? i : r1 - 1);
		}
#pragma unroll
		for (int u = 0; u < U; ++u) {
			const int64_t i = i0 + (int64_t)u * nt;
			if (i < r1)
				store(i, t[u]);
		}
	}
}

// Row sums s_i = sum_k a(i, k) v[k] for the rows r0 + tid, r0 + tid + nt,
// ... of one system, in column order (the same bits either way), handed to
// f(i, s_i): from the grid-stencil arrays when the batch has them (no index
// is read: the coefficient and neighbour loads of a batch of rows are all
// independent), else from the CSR.
template<class V, int U, class F>
__device__ __forceinline__ void row_sums(const BatchArgs &a, const V *val, const V *gd, const V *gu1,
                                         const V *gu2, const V *__restrict__ v, int sys,
                                         int64_t R0, int64_t r0, int64_t r1, int tid, int nt, F &&f) {
	if (a.side && U == 1) {
		const int sd = a.side[sys];
		for (int64_t i = r0 + tid; i < r1; i += nt) {
			const int l = (int)(i - R0), ii = l % sd, jj = l / sd;
			V sum = V(0);
			if (jj > 0)
				sum = fmav(gu2[i - sd], v[i - sd], sum);
			if (ii > 0)
				sum = fmav(gu1[i - 1], v[i - 1], sum);
			sum = fmav(gd[i], v[i], sum);
			if (ii < sd - 1)
				sum = fmav(gu1[i], v[i + 1], sum);
			if (jj < sd - 1)
				sum = fmav(gu2[i], v[i + sd], sum);
			f(i, sum);
		}
	}
	else if (a.side) {
		const int sd = a.side[sys];
		rows_batched<U>(
			r0, r1, tid, nt,
			[&](int64_t i) {
				// every load from an address inside the system (an absent
				// neighbour reads row i and its term is not added), so none
				// waits on a branch
				const int l = (int)(i - R0), ii = l % sd, jj = l / sd;
				const bool s_lo = jj > 0, w_lo = ii > 0, w_hi = ii < sd - 1, s_hi = jj < sd - 1;
				const int64_t is = s_lo ? i - sd : i, iw = w_lo ? i - 1 : i;
				const int64_t ie = w_hi ? i + 1 : i, in = s_hi ? i + sd : i;
				const V c0 = gu2[is], x0 = v[is], c1 = gu1[iw], x1 = v[iw], c2 = gd[i], x2 = v[i];
				const V c3 = gu1[i], x3 = v[ie], c4 = gu2[i], x4 = v[in];
				V sum = V(0);
				sum = s_lo ? fmav(c0, x0, sum) : sum;
				sum = w_lo ? fmav(c1, x1, sum) : sum;
				sum = fmav(c2, x2, sum);
				sum = w_hi ? fmav(c3, x3, sum) : sum;
				sum = s_hi ? fmav(c4, x4, sum) : sum;
				return sum;
			},
			f);
	}
	else {
		for (int64_t i = r0 + tid; i < r1; i += nt) {
			V sum = V(0);
			for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k)
				sum = fmav(val[k], v[a.col[k]], sum);
			f(i, sum);
		}
	}
}

// sum of NV doubles over the cluster: every CTA block-reduces its values,
// publishes them in its shared slot for phase `ph`, and after the cluster
// barrier reads all CTAs' slots in rank order
template<int NV>
__device__ __forceinline__ void cluster_sum(double (&v)[NV], double *sh_tree,
                                            double (*slots)[4], int ph, cgrp::cluster_group &cl) {
	block_sum<NV>(v, sh_tree);
	if (threadIdx.x == 0)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			slots[ph & 1][k] = v[k];
	__threadfence();
	cl.sync();
	double t[NV];
#pragma unroll
	for (int k = 0; k < NV; ++k)
		t[k] = 0.0;
	for (unsigned r = 0; r < cl.num_blocks(); ++r) {
		double(*rs)[4] = cl.map_shared_rank(slots, r);
#pragma unroll
		for (int k = 0; k < NV; ++k)
			t[k] += rs[ph & 1][k];
	}
#pragma unroll
	for (int k = 0; k < NV; ++k)
		v[k] = t[k];
}

// sum over the team: the cluster (team > 1) or the CTA alone (team == 1)
template<int NV>
__device__ __forceinline__ void team_sum(double (&v)[NV], double *sh_tree, double (*slots)[4],
                                         int ph, cgrp::cluster_group &cl, int team) {
	if (team > 1) {
		cluster_sum<NV>(v, sh_tree, slots, ph, cl);
		return;
	}
	block_sum<NV>(v, sh_tree);
	if (threadIdx.x == 0)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			slots[ph & 1][k] = v[k];
	__syncthreads();
#pragma unroll
	for (int k = 0; k < NV; ++k)
		v[k] = slots[ph & 1][k];
}

// the team's writes to global memory visible to the whole team
__device__ __forceinline__ void team_sync(cgrp::cluster_group &cl, int team) {
	__threadfence();
	if (team > 1)
		cl.sync();
	else
		__syncthreads();
}

// MAXT: the largest CTA the kernel is built for, MINB CTAs of it resident
// on an SM; U32: FP32 rows per batch of the row loops (FP64: half).  One
// 1024-thread CTA an SM leaves 64 registers a thread (one row at a time).
template<int MAXT, int MINB, int U32>
__global__ void __launch_bounds__(MAXT, MINB)
k_batch_cg(BatchArgs a) {
	constexpr int U64 = U32 > 1 ? U32 / 2 : 1;
	cgrp::cluster_group cl = cgrp::this_cluster();
	const int crank = (int)cl.block_rank();
	const int csize = (int)cl.num_blocks();
	const int cidx = (int)(blockIdx.x / csize);
	// clusters 0..nbig-1: one system each (team = the cluster); then one
	// system per CTA (team = 1); the choice is uniform across a cluster
	const bool whole = cidx < a.nbig;
	const int team = whole ? csize : 1;
	const int trank = whole ? crank : 0;
	const int slot = whole ? cidx : a.nbig + (cidx - a.nbig) * csize + crank;
	if (slot >= a.nsys)
		return;  // a CTA of the last cluster with no system (team 1 only)
	const int sys = a.order[slot];
	const int64_t R0 = a.off[sys], R1 = a.off[sys + 1];
	const int64_t nrow = R1 - R0;
	const int64_t chunk = (nrow + team - 1) / team;
	const int64_t lo = chunk * trank, hi = chunk * (trank + 1);
	const int64_t r0 = R0 + (lo < nrow ? lo : nrow);
	const int64_t r1 = R0 + (hi < nrow ? hi : nrow);
	__shared__ double sh_tree[4 * 32];
	__shared__ double slots[2][4];
	int ph = 0;
	const int tid = threadIdx.x, nt = blockDim.x;

	// ||b|| and the initial residual (FP64): r = b - A x (or b), x32 = 0
	double v2[2] = {0.0, 0.0};
	for (int64_t i = r0 + tid; i < r1; i += nt) {
		const double bi = a.b[i];
		v2[0] = fma(bi, bi, v2[0]);
		if (a.zero_guess)
			a.x[i] = 0.0;
		v2[1] = fma(a.x[i], a.x[i], v2[1]);
		a.x32[i] = 0.f;
	}
	team_sum<2>(v2, sh_tree, slots, ph++, cl, team);
	double bnorm = sqrt(v2[0]);
	const double rhs_norm = bnorm;
	if (bnorm == 0.0)
		bnorm = 1.0;
	const double tol = (double)a.rtol * bnorm;
	const double sol0 = sqrt(v2[1]);

	// FP64 residual replacement: r64 = b - A64 x, r32 = (float) r64; returns
	// ||r64|| and r32 . D^-1 r32 (all CTAs of the cluster get the same)
	auto replace = [&](double &res, double &rz) {
		double t[2] = {0.0, 0.0};
		row_sums<double, U64>(a, a.val64, a.gd64, a.gu1_64, a.gu2_64, a.x, sys, R0, r0, r1, tid, nt,
		                 [&](int64_t i, double s) {
			                 const double ri = a.b[i] - s;
			                 const float r32 = (float)ri;
			                 a.r32[i] = r32;
			                 t[0] = fma(ri, ri, t[0]);
			                 t[1] = fma((double)r32, (double)(a.dinv32[i] * r32), t[1]);
		                 });
		team_sum<2>(t, sh_tree, slots, ph++, cl, team);
		res = sqrt(t[0]);
		rz = t[1];
	};
	double res = 0.0, rz = 0.0;
	replace(res, rz);
	const double res0 = res;
	double rmax = res;
	int status = FS_DIVERGED_ITERS;
	int iters = 0, outer = 0;
	bool fp32_start = true;  // the FP32 loop starts from r32 (no FP64 head ran)
	double rho = rz;
	if (res >= tol && a.head > 0.0 && res >= a.head * bnorm && a.maxiter > 0) {
		// FP64 head (the cg_apply64 iteration): r64 = b - A x, p = D^-1 r
		double t[1] = {0.0};
		row_sums<double, U64>(a, a.val64, a.gd64, a.gu1_64, a.gu2_64, a.x, sys, R0, r0, r1, tid, nt,
		                 [&](int64_t i, double sum) {
			                 const double ri = a.b[i] - sum;
			                 a.r64[i] = ri;
			                 const double zi = a.dinv64[i] * ri;
			                 a.p64[i] = zi;
			                 t[0] = fma(ri, zi, t[0]);
		                 });
		team_sum<1>(t, sh_tree, slots, ph++, cl, team);
		rho = t[0];
		double rho_old = rho;
		bool switch_now = false;
		for (int it = 0; it < a.maxiter; ++it) {
			double q[1] = {0.0};
			row_sums<double, U64>(a, a.val64, a.gd64, a.gu1_64, a.gu2_64, a.p64, sys, R0, r0, r1, tid, nt,
			                 [&](int64_t i, double sum) {
				                 a.w64[i] = sum;
				                 q[0] = fma(sum, a.p64[i], q[0]);
			                 });
			team_sum<1>(q, sh_tree, slots, ph++, cl, team);
			const double alpha = rho / q[0];
			double u[2] = {0.0, 0.0};
			struct H5 { double x, p, w, r, d; };
			rows_batched<U64>(
				r0, r1, tid, nt,
				[&](int64_t i) { return H5{a.x[i], a.p64[i], a.w64[i], a.r64[i], a.dinv64[i]}; },
				[&](int64_t i, const H5 &h) {
					a.x[i] = fma(alpha, h.p, h.x);
					const double ri = fma(-alpha, h.w, h.r);
					a.r64[i] = ri;
					u[0] = fma(ri, ri, u[0]);
					u[1] = fma(ri, h.d * ri, u[1]);
				});
			team_sum<2>(u, sh_tree, slots, ph++, cl, team);
			iters = it + 1;
			res = sqrt(u[0]);
			if (res < tol) {
				status = FS_CONVERGED_RTOL;
				break;
			}
			if (!isfinite(res) || iters >= a.maxiter)
				break;
			rho_old = rho;
			rho = u[1];
			if (res < a.head * bnorm) {
				switch_now = true;
				break;
			}
			const double beta = rho / rho_old;
			rows_batched<U64>(
				r0, r1, tid, nt, [&](int64_t i) { return make_double3(a.p64[i], a.dinv64[i], a.r64[i]); },
				[&](int64_t i, const double3 &h) { a.p64[i] = fma(beta, h.x, h.y * h.z); });
			team_sync(cl, team);
		}
		if (switch_now) {
			// the same Krylov process continues in FP32: r replaced by the
			// FP64 b - A x, the direction p = z + beta p from the last FP64 rho
			team_sync(cl, team);
			double rz32 = 0.0;
			replace(res, rz32);
			++outer;
			rmax = res;
			if (res < tol)
				status = FS_CONVERGED_RTOL;
			const float bf = (float)(rz32 / rho_old);
			rho = rz32;
			for (int64_t i = r0 + tid; i < r1; i += nt)
				a.p32[i] = fmaf(bf, (float)a.p64[i], a.dinv32[i] * a.r32[i]);
			team_sync(cl, team);
			fp32_start = false;
		}
		else if (status != FS_CONVERGED_RTOL) {
			fp32_start = false;
			iters = a.maxiter;  // stopped by maxiter or a non-finite residual
		}
	}
	if (res < tol) {
		status = FS_CONVERGED_RTOL;
	}
	else if (iters < a.maxiter) {
		if (fp32_start) {
			// p = D^-1 r, rho = r . z
			for (int64_t i = r0 + tid; i < r1; i += nt)
				a.p32[i] = a.dinv32[i] * a.r32[i];
			rho = rz;
			team_sync(cl, team);
		}
		for (int it = iters; it < a.maxiter; ++it) {
			// w = A p, p . w
			// the FP32 phase's dots: exact FP32 products summed in compensated
			// FP32 pairs per thread (FP64 accuracy without the FP64 pipe, which
			// runs at 1/64 of the FP32 rate), FP64 across the team
			cf32 cq{0.f, 0.f};
			row_sums<float, U32>(a, a.val32, a.gd32, a.gu1_32, a.gu2_32, a.p32, sys, R0, r0, r1, tid, nt,
			                [&](int64_t i, float s) {
				                a.w32[i] = s;
				                cq.add_prod(s, a.p32[i]);
			                });
			double q[1] = {(double)cq.hi + (double)cq.lo};
			team_sum<1>(q, sh_tree, slots, ph++, cl, team);
			const double alpha = rho / q[0];
			const float af = (float)alpha;
			// x32 += alpha p, r -= alpha w, ||r||^2, r . z
			cf32 cu0{0.f, 0.f}, cu1{0.f, 0.f};
			struct S5 { float x, p, w, r, d; };
			rows_batched<U32>(
				r0, r1, tid, nt,
				[&](int64_t i) { return S5{a.x32[i], a.p32[i], a.w32[i], a.r32[i], a.dinv32[i]}; },
				[&](int64_t i, const S5 &h) {
					a.x32[i] = fmaf(af, h.p, h.x);
					const float ri = fmaf(-af, h.w, h.r);
					a.r32[i] = ri;
					cu0.add_prod(ri, ri);
					cu1.add_prod(ri, h.d * ri);
				});
			double u[2] = {(double)cu0.hi + (double)cu0.lo, (double)cu1.hi + (double)cu1.lo};
			team_sum<2>(u, sh_tree, slots, ph++, cl, team);
			iters = it + 1;
			double est = sqrt(u[0]);
			double rz_new = u[1];
			const bool last = iters >= a.maxiter;
			if (est < a.delta * rmax || est < tol || last || !isfinite(est)) {
				// fold the correction and replace r by the FP64 residual
				for (int64_t i = r0 + tid; i < r1; i += nt) {
					a.x[i] += (double)a.x32[i];
					a.x32[i] = 0.f;
				}
				team_sync(cl, team);
				replace(res, rz_new);
				++outer;
				rmax = res;
				if (res < tol) {
					status = FS_CONVERGED_RTOL;
					break;
				}
				if (last || !isfinite(res))
					break;
			}
			else {
				res = est;
			}
			const double beta = rz_new / rho;
			rho = rz_new;
			const float bf = (float)beta;
			rows_batched<U32>(
				r0, r1, tid, nt, [&](int64_t i) { return make_float3(a.p32[i], a.dinv32[i], a.r32[i]); },
				[&](int64_t i, const float3 &h) { a.p32[i] = fmaf(bf, h.x, h.y * h.z); });
			team_sync(cl, team);
		}
	}
	double xn[1] = {0.0};
	for (int64_t i = r0 + tid; i < r1; i += nt)
		xn[0] = fma(a.x[i], a.x[i], xn[0]);
	team_sum<1>(xn, sh_tree, slots, ph++, cl, team);
	if (trank == 0 && tid == 0) {
		fs_solve_info inf;
		inf.status = status;
		inf.iters = status == FS_CONVERGED_RTOL ? iters : 0;
		inf.restarts = outer;
		inf.res_norm_initial = (float)res0;
		inf.res_norm_final = (float)res;
		inf.sol_norm_initial = a.zero_guess ? 0.f : (float)sol0;
		inf.sol_norm_final = (float)sqrt(xn[0]);
		inf.rhs_norm = (float)rhs_norm;
		a.info[sys] = inf;
	}
	// no CTA may leave while a peer can still read its shared slots
	if (team > 1)
		cl.sync();
}

// The grid-stencil storage of a batch, one thread per row: row i of system
// k (side s, local row l = ii + s jj) must hold exactly the columns
// i - s, i - 1, i, i + 1, i + s that lie inside the s x s grid, in that
// order, and its lower entries must equal their partners a(i - s, i),
// a(i - 1, i) bit for bit; any other row sets *bad.  Writes a(i, i),
// a(i, i + 1), a(i, i + s) (0 where absent) in FP64 and FP32 at g + {0, ld,
// 2 ld} + i.
__global__ void k_batch_grid_build(int64_t n, int nsys, const int64_t *__restrict__ off,
                                   const int *__restrict__ side, const int *__restrict__ rp,
                                   const int *__restrict__ col, const double *__restrict__ val,
                                   double *g64, float *g32, int64_t ld, unsigned *bad) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x) {
		// the system holding row i: the last k with off[k] <= i
		int lo = 0, hi = nsys;
		while (hi - lo > 1) {
			const int mid = (lo + hi) / 2;
			if (off[mid] <= i)
				lo = mid;
			else
				hi = mid;
		}
		const int64_t sd = side[lo];
		const int64_t l = i - off[lo], ii = l % sd, jj = l / sd;
		int k = rp[i];
		const int e = rp[i + 1];
		bool ok = true;
		double d = 0.0, u1 = 0.0, u2 = 0.0;
		if (jj > 0) {
			// partner a(i - s, i): the last entry of row i - s
			const int q = rp[i - sd + 1] - 1;
			ok = k < e && col[k] == i - sd && q >= rp[i - sd] &&
			     __double_as_longlong(val[k]) == __double_as_longlong(val[q]);
			++k;
		}
		if (ok && ii > 0) {
			// partner a(i - 1, i): row i - 1's entry after its diagonal
			const int q = rp[i - 1] + (jj > 0) + (ii > 1) + 1;
			ok = k < e && col[k] == i - 1 && q < rp[i] &&
			     __double_as_longlong(val[k]) == __double_as_longlong(val[q]);
			++k;
		}
		if (ok) {
			ok = k < e && col[k] == i;
			if (ok)
				d = val[k];
			++k;
		}
		if (ok && ii < sd - 1) {
			ok = k < e && col[k] == i + 1;
			if (ok)
				u1 = val[k];
			++k;
		}
		if (ok && jj < sd - 1) {
			ok = k < e && col[k] == i + sd;
			if (ok)
				u2 = val[k];
			++k;
		}
		if (!ok || k != e)
			atomicOr(bad, 1u);
		g64[i] = d;
		g64[ld + i] = u1;
		g64[2 * ld + i] = u2;
		g32[i] = (float)d;
		g32[ld + i] = (float)u1;
		g32[2 * ld + i] = (float)u2;
	}
}

struct BatchPlan {
	std::vector<int64_t> off;
	int64_t *d_off = nullptr;
	int *d_order = nullptr;
	fs_solve_info *d_info = nullptr;
	float *work = nullptr;  // x32, r32, p32, w32
	double *work64 = nullptr;  // r64, p64, w64 of the FP64 head
	int nsys = 0;
	int tuned_cluster = 0, tuned_threads = 0;
	int tuned_nbig = -1;  // systems that own a whole cluster (-1: all)
	// grid-stencil storage (every system a 5-point s x s grid with symmetric
	// values): per-system sides, diagonal and upper diagonals; `grid` is 1
	// when it holds for the values of generation `grid_gen`, 0 when not, -1
	// not checked
	int *d_side = nullptr;
	double *g64 = nullptr;
	float *g32 = nullptr;
	unsigned *d_bad = nullptr;
	int grid = -1;
	unsigned grid_gen = 0;
};

void free_plan(BatchPlan &p) {
	for (void *q : {(void *)p.d_off, (void *)p.d_order, (void *)p.d_info, (void *)p.work,
	                (void *)p.work64, (void *)p.d_side, (void *)p.g64, (void *)p.g32, (void *)p.d_bad})
		if (q)
			cudaFree(q);
}

// one plan per (matrix, partition); freed with the matrix
std::map<std::pair<const Csr *, std::vector<int64_t>>, BatchPlan> g_plans;

// (re)check the batch for the grid-stencil storage after a change of values
int ensure_batch_grid(Ctx *ctx, const Csr *A, BatchPlan &p) {
	if (p.grid >= 0 && p.grid_gen == A->values_gen)
		return FS_OK;
	p.grid = 0;
	p.grid_gen = A->values_gen;
	const int nsys = p.nsys;
	std::vector<int> side(nsys);
	for (int k = 0; k < nsys; ++k) {
		const int64_t m = p.off[k + 1] - p.off[k];
		int64_t sd = (int64_t)std::llround(std::sqrt((double)m));
		while (sd * sd > m)
			--sd;
		while ((sd + 1) * (sd + 1) <= m)
			++sd;
		if (sd * sd != m || sd > 46340)
			return FS_OK;  // not a square grid: the CSR row loops
		side[k] = (int)sd;
	}
	const size_t n = (size_t)A->nrows, ld = n + 32;
	if (!p.d_side) {
		FS_CUDA_TRY(ctx, cudaMalloc(&p.d_side, sizeof(int) * nsys));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.g64, sizeof(double) * 3 * ld));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.g32, sizeof(float) * 3 * ld));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.d_bad, sizeof(unsigned)));
	}
	FS_CUDA_TRY(ctx, cudaMemcpy(p.d_side, side.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice));
	FS_CUDA_TRY(ctx, cudaMemsetAsync(p.d_bad, 0, sizeof(unsigned), ctx->stream));
	if (n > 0) {
		k_batch_grid_build<<<grid_for(ctx, (int64_t)n, 256, 4), 256, 0, ctx->stream>>>(
			(int64_t)n, nsys, p.d_off, p.d_side, A->rowptr, A->col, A->val, p.g64, p.g32,
			(int64_t)ld, p.d_bad);
		FS_TRY(check_launch(ctx, "batched grid-stencil build"));
	}
	unsigned bad = 1;
	FS_CUDA_TRY(ctx, cudaMemcpyAsync(&bad, p.d_bad, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
	FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	p.grid = bad ? 0 : 1;
	return FS_OK;
}

// a.nbig systems own a cluster each; the rest take one CTA each, `cluster`
// of them per cluster
int launch_batch(Ctx *ctx, const BatchArgs &a, int nsys, int cluster, int threads) {
	const int nclusters = a.nbig + (nsys - a.nbig + cluster - 1) / cluster;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)(nclusters * cluster), 1, 1);
	cfg.blockDim = dim3((unsigned)threads, 1, 1);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = ctx->stream;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = (unsigned)cluster;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	cudaError_t e = threads > 512   ? cudaLaunchKernelEx(&cfg, k_batch_cg<1024, 1, 1>, a)
	                : threads > 256 ? cudaLaunchKernelEx(&cfg, k_batch_cg<512, 1, 4>, a)
	                                : cudaLaunchKernelEx(&cfg, k_batch_cg<256, 2, 8>, a);
	if (e != cudaSuccess)
		return set_err(ctx, FS_ERR_CUDA, "batched CG launch (cluster %d, %d threads): %s", cluster,
		               threads, cudaGetErrorString(e));
	ctx->launches++;
	return FS_OK;
}

// cluster_systems: -1 chooses (with the sizes), else that many of the
// largest systems own a cluster and the rest one CTA each
int batch_solve(fs_ctx h, const fs_krylov_settings *s, fs_csr Ah, int nsys, const int64_t *sys_offsets,
                fs_vec bh, fs_vec xh, int cluster_size, int threads, int cluster_systems,
                fs_solve_info *infos) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Csr *A = reinterpret_cast<Csr *>(Ah);
	Vec *b = reinterpret_cast<Vec *>(bh), *x = reinterpret_cast<Vec *>(xh);
	if (!ok_ctx(ctx) || !ok_csr(A) || !ok_vec(b) || !ok_vec(x) || !s || !sys_offsets || !infos)
		return FS_ERR_BAD_HANDLE;
	FS_TRY(reject_matrix_free(A, "fs_batch_cg_solve"));
	if (nsys < 1 || sys_offsets[0] != 0 || sys_offsets[nsys] != A->nrows || A->nrows != A->ncols ||
	    b->n != A->nrows || x->n != A->nrows || b->dtype != FS_F64 || x->dtype != FS_F64)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_batch_cg_solve: offsets/sizes do not match");
	if (cluster_size != 0 && (cluster_size < 1 || cluster_size > 8 ||
	                          (cluster_size & (cluster_size - 1))))
		return set_err(ctx, FS_ERR_INVALID_ARG, "cluster_size must be 0 (autotune), 1, 2, 4 or 8");
	if (threads != 0 && (threads < 64 || threads > 1024 || threads % 32))
		return set_err(ctx, FS_ERR_INVALID_ARG, "threads must be 0 (autotune) or 64..1024, a multiple of 32");
	cudaSetDevice(ctx->device);
	std::vector<int64_t> off(sys_offsets, sys_offsets + nsys + 1);
	for (int k = 0; k < nsys; ++k)
		if (off[k + 1] < off[k])
			return set_err(ctx, FS_ERR_INVALID_ARG, "fs_batch_cg_solve: offsets not monotone");
	auto key = std::make_pair((const Csr *)A, off);
	auto it = g_plans.find(key);
	if (it == g_plans.end()) {
		// check block-diagonality once per partition
		std::vector<int> hc(A->nnz);
		FS_CUDA_TRY(ctx, cudaMemcpy(hc.data(), A->col, A->nnz * sizeof(int), cudaMemcpyDeviceToHost));
		for (int k = 0; k < nsys; ++k)
			for (int64_t r = off[k]; r < off[k + 1]; ++r)
				for (int q = A->h_rowptr[r]; q < A->h_rowptr[r + 1]; ++q)
					if (hc[q] < off[k] || hc[q] >= off[k + 1])
						return set_err(ctx, FS_ERR_INVALID_ARG,
						               "fs_batch_cg_solve: row %lld couples outside system %d",
						               (long long)r, k);
		BatchPlan p;
		p.off = off;
		p.nsys = nsys;
		// largest systems first (longest-processing-time order)
		std::vector<int> order(nsys);
		std::iota(order.begin(), order.end(), 0);
		std::stable_sort(order.begin(), order.end(), [&](int i, int j) {
			return off[i + 1] - off[i] > off[j + 1] - off[j];
		});
		const size_t n = (size_t)A->nrows;
		FS_CUDA_TRY(ctx, cudaMalloc(&p.d_off, sizeof(int64_t) * (nsys + 1)));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.d_order, sizeof(int) * nsys));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.d_info, sizeof(fs_solve_info) * nsys));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.work, sizeof(float) * 4 * (n + 32)));
		FS_CUDA_TRY(ctx, cudaMalloc(&p.work64, sizeof(double) * 3 * (n + 32)));
		FS_CUDA_TRY(ctx, cudaMemcpy(p.d_off, off.data(), sizeof(int64_t) * (nsys + 1), cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, cudaMemcpy(p.d_order, order.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice));
		FS_CUDA_TRY(ctx, fence_setup_copies());
		it = g_plans.emplace(key, p).first;
	}
	BatchPlan &p = it->second;
	FS_TRY(ensure_val32(A));
	FS_TRY(ensure_dinv(A));
	FS_TRY(ensure_batch_grid(ctx, A, p));
	const size_t n = (size_t)A->nrows;
	BatchArgs a;
	a.nsys = nsys;
	a.order = p.d_order;
	a.off = p.d_off;
	a.rowptr = A->rowptr;
	a.col = A->col;
	a.val32 = A->val32;
	a.val64 = A->val;
	a.dinv32 = A->dinv32;
	a.dinv64 = A->dinv;
	a.b = (const double *)b->d;
	a.x = (double *)x->d;
	a.x32 = p.work;
	a.r32 = p.work + (n + 32);
	a.p32 = p.work + 2 * (n + 32);
	a.w32 = p.work + 3 * (n + 32);
	a.r64 = p.work64;
	a.p64 = p.work64 + (n + 32);
	a.w64 = p.work64 + 2 * (n + 32);
	a.head = s->fp64_head > (double)s->base.rtol ? s->fp64_head : 0.0;
	a.info = p.d_info;
	a.maxiter = s->base.maxiter;
	a.rtol = s->base.rtol;
	a.delta = s->inner_rtol > 0 ? s->inner_rtol : 0.1;
	a.zero_guess = s->base.use_zero_guess ? 1 : 0;
	a.nbig = cluster_systems >= 0 ? cluster_systems : nsys;
	a.side = nullptr;
	a.gd64 = a.gu1_64 = a.gu2_64 = nullptr;
	a.gd32 = a.gu1_32 = a.gu2_32 = nullptr;
	if (p.grid == 1) {
		const size_t ld = n + 32;
		a.side = p.d_side;
		a.gd64 = p.g64;
		a.gu1_64 = p.g64 + ld;
		a.gu2_64 = p.g64 + 2 * ld;
		a.gd32 = p.g32;
		a.gu1_32 = p.g32 + ld;
		a.gu2_32 = p.g32 + 2 * ld;
	}

	int cl = cluster_size, th = threads;
	if (cl == 0 || th == 0) {
		if (p.tuned_cluster == 0) {
			// autotuner, stage 1: time a short capped run of each cluster /
			// CTA size (every system a whole cluster) on this batch and keep
			// the fastest cluster size for each CTA size; the solution is
			// restored afterwards
			std::vector<double> xsave(n);
			FS_CUDA_TRY(ctx, cudaMemcpy(xsave.data(), x->d, n * 8, cudaMemcpyDeviceToHost));
			BatchArgs t = a;
			t.maxiter = std::min(a.maxiter, 40);
			t.zero_guess = 1;
			t.nbig = nsys;
			const int tsizes[3] = {256, 512, 1024};
			float best_t[3] = {1e30f, 1e30f, 1e30f};
			int best_c[3] = {0, 0, 0};
			cudaEvent_t e0, e1;
			cudaEventCreate(&e0);
			cudaEventCreate(&e1);
			auto time_launch = [&](const BatchArgs &args, int c, int tt, float &ms) {
				cudaEventRecord(e0, ctx->stream);
				int st = launch_batch(ctx, args, nsys, c, tt);
				cudaEventRecord(e1, ctx->stream);
				if (st != FS_OK) {
					cudaGetLastError();
					return false;
				}
				cudaEventSynchronize(e1);
				cudaEventElapsedTime(&ms, e0, e1);
				return true;
			};
			for (int ti = 0; ti < 3; ++ti)
				for (int c : {1, 2, 4, 8}) {
					if ((cluster_size && c != cluster_size) || (threads && tsizes[ti] != threads))
						continue;
					float ms = 0;
					if (time_launch(t, c, tsizes[ti], ms) && ms < best_t[ti]) {
						best_t[ti] = ms;
						best_c[ti] = c;
					}
				}
			float best = 1e30f;
			for (int ti = 0; ti < 3; ++ti)
				if (best_c[ti] && best_t[ti] < best) {
					best = best_t[ti];
					p.tuned_cluster = best_c[ti];
					p.tuned_threads = tsizes[ti];
				}
			if (p.tuned_cluster == 0) {
				cudaEventDestroy(e0);
				cudaEventDestroy(e1);
				return set_err(ctx, FS_ERR_CUDA, "batched CG: no launch configuration ran");
			}
			// stage 2 (only when the caller fixed neither size): complete
			// solves -- capped runs see neither that the largest systems
			// need the most iterations nor how the FP64 head and the FP32
			// phase share the time -- of each CTA size's stage-1 winner,
			// against splits where the largest systems own a cluster and the
			// rest one CTA each
			p.tuned_nbig = nsys;
			if (!cluster_size && !threads && nsys >= 8) {
				struct Cand { int c, t, nbig; };
				std::vector<Cand> cands;
				for (int ti = 0; ti < 3; ++ti)
					if (best_c[ti])
						cands.push_back({best_c[ti], tsizes[ti], nsys});
				cands.push_back({2, 512, std::max(1, nsys / 16)});
				cands.push_back({4, 1024, std::max(1, nsys / 32)});
				BatchArgs f = a;
				f.zero_guess = 1;
				float best2 = 1e30f;
				for (const Cand &cd : cands) {
					f.nbig = cd.nbig;
					float ms = 0;
					if (time_launch(f, cd.c, cd.t, ms) && ms < best2) {
						best2 = ms;
						p.tuned_cluster = cd.c;
						p.tuned_threads = cd.t;
						p.tuned_nbig = cd.nbig;
					}
				}
			}
			cudaEventDestroy(e0);
			cudaEventDestroy(e1);
			FS_CUDA_TRY(ctx, cudaMemcpy(x->d, xsave.data(), n * 8, cudaMemcpyHostToDevice));
			FS_CUDA_TRY(ctx, fence_setup_copies());
		}
		if (!cl)
			cl = p.tuned_cluster;
		if (!th)
			th = p.tuned_threads;
		if (!cluster_size && !threads && p.tuned_nbig >= 0 && cluster_systems < 0)
			a.nbig = p.tuned_nbig;
	}
	FS_TRY(launch_batch(ctx, a, nsys, cl, th));
	FS_CUDA_TRY(ctx, cudaMemcpyAsync(infos, p.d_info, sizeof(fs_solve_info) * nsys, cudaMemcpyDeviceToHost,
	                                 ctx->stream));
	FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	return FS_OK;
}

}  // namespace

void destroy_batch_plans(const Csr *A) {
	for (auto it = g_plans.begin(); it != g_plans.end();) {
		if (it->first.first == A) {
			free_plan(it->second);
			it = g_plans.erase(it);
		}
		else {
			++it;
		}
	}
}

}  // namespace fsg

using namespace fsg;

extern "C" FS_API int fs_batch_cg_solve(fs_ctx h, const fs_krylov_settings *s, fs_csr A, int nsys,
                                        const int64_t *sys_offsets, fs_vec b, fs_vec x,
                                        int cluster_size, int threads, fs_solve_info *infos) {
	return batch_solve(h, s, A, nsys, sys_offsets, b, x, cluster_size, threads, -1, infos);
}

extern "C" FS_API int fs_batch_cg_solve_split(fs_ctx h, const fs_krylov_settings *s, fs_csr A,
                                              int nsys, const int64_t *sys_offsets, fs_vec b,
                                              fs_vec x, int cluster_size, int threads,
                                              int cluster_systems, fs_solve_info *infos) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(ctx))
		return FS_ERR_BAD_HANDLE;
	if (cluster_size == 0 || threads == 0 || cluster_systems < 0 || cluster_systems > nsys)
		return set_err(ctx, FS_ERR_INVALID_ARG,
		               "fs_batch_cg_solve_split: explicit sizes and 0 <= cluster_systems <= nsys");
	return batch_solve(h, s, A, nsys, sys_offsets, b, x, cluster_size, threads, cluster_systems, infos);
}

extern "C" FS_API int fs_batch_tuning(fs_ctx h, fs_csr Ah, int nsys, const int64_t *sys_offsets,
                                      int *cluster_size, int *threads) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Csr *A = reinterpret_cast<Csr *>(Ah);
	if (!ok_ctx(ctx) || !ok_csr(A) || !sys_offsets || !cluster_size || !threads)
		return FS_ERR_BAD_HANDLE;
	std::vector<int64_t> off(sys_offsets, sys_offsets + nsys + 1);
	auto it = g_plans.find(std::make_pair((const Csr *)A, off));
	if (it == g_plans.end())
		return set_err(ctx, FS_ERR_INVALID_ARG, "no batched solve has run on this partition");
	*cluster_size = it->second.tuned_cluster;
	*threads = it->second.tuned_threads;
	return FS_OK;
}

extern "C" FS_API int fs_batch_schedule(fs_ctx h, fs_csr Ah, int nsys, const int64_t *sys_offsets,
                                        int *cluster_size, int *threads, int *cluster_systems) {
	FS_TRY(fs_batch_tuning(h, Ah, nsys, sys_offsets, cluster_size, threads));
	if (!cluster_systems)
		return FS_ERR_BAD_HANDLE;
	Csr *A = reinterpret_cast<Csr *>(Ah);
	std::vector<int64_t> off(sys_offsets, sys_offsets + nsys + 1);
	const int nbig = g_plans.find(std::make_pair((const Csr *)A, off))->second.tuned_nbig;
	*cluster_systems = nbig < 0 ? nsys : nbig;
	return FS_OK;
}

extern "C" FS_API int fs_batch_format(fs_ctx h, fs_csr Ah, int nsys, const int64_t *sys_offsets,
                                      int *format) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Csr *A = reinterpret_cast<Csr *>(Ah);
	if (!ok_ctx(ctx) || !ok_csr(A) || !sys_offsets || !format || nsys < 1)
		return FS_ERR_BAD_HANDLE;
	std::vector<int64_t> off(sys_offsets, sys_offsets + nsys + 1);
	auto it = g_plans.find(std::make_pair((const Csr *)A, off));
	if (it == g_plans.end())
		return set_err(ctx, FS_ERR_INVALID_ARG, "no batched solve has run on this partition");
	*format = it->second.grid == 1 ? FS_BATCH_GRID : FS_BATCH_CSR;
	return FS_OK;
}
