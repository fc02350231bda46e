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
// more iterations), then FP32 values and vectors, dots accumulated in FP64;
// the residual is replaced by the FP64 one, b - A x with the FP64 values,
// whenever it has dropped by `delta` and at every stop, and the stopping test
// is on that FP64 residual.
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
};

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

__global__ void __launch_bounds__(1024)
k_batch_cg(BatchArgs a) {
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
		for (int64_t i = r0 + tid; i < r1; i += nt) {
			double s = 0.0;
			for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k)
				s = fma(a.val64[k], a.x[a.col[k]], s);
			const double ri = a.b[i] - s;
			const float r32 = (float)ri;
			a.r32[i] = r32;
			t[0] = fma(ri, ri, t[0]);
			t[1] = fma((double)r32, (double)(a.dinv32[i] * r32), t[1]);
		}
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
		for (int64_t i = r0 + tid; i < r1; i += nt) {
			double sum = 0.0;
			for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k)
				sum = fma(a.val64[k], a.x[a.col[k]], sum);
			const double ri = a.b[i] - sum;
			a.r64[i] = ri;
			const double zi = a.dinv64[i] * ri;
			a.p64[i] = zi;
			t[0] = fma(ri, zi, t[0]);
		}
		team_sum<1>(t, sh_tree, slots, ph++, cl, team);
		rho = t[0];
		double rho_old = rho;
		bool switch_now = false;
		for (int it = 0; it < a.maxiter; ++it) {
			double q[1] = {0.0};
			for (int64_t i = r0 + tid; i < r1; i += nt) {
				double sum = 0.0;
				for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k)
					sum = fma(a.val64[k], a.p64[a.col[k]], sum);
				a.w64[i] = sum;
				q[0] = fma(sum, a.p64[i], q[0]);
			}
			team_sum<1>(q, sh_tree, slots, ph++, cl, team);
			const double alpha = rho / q[0];
			double u[2] = {0.0, 0.0};
			for (int64_t i = r0 + tid; i < r1; i += nt) {
				a.x[i] = fma(alpha, a.p64[i], a.x[i]);
				const double ri = fma(-alpha, a.w64[i], a.r64[i]);
				a.r64[i] = ri;
				u[0] = fma(ri, ri, u[0]);
				u[1] = fma(ri, a.dinv64[i] * ri, u[1]);
			}
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
			for (int64_t i = r0 + tid; i < r1; i += nt)
				a.p64[i] = fma(beta, a.p64[i], a.dinv64[i] * a.r64[i]);
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
			double q[1] = {0.0};
			for (int64_t i = r0 + tid; i < r1; i += nt) {
				float s = 0.f;
				for (int k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k)
					s = fmaf(a.val32[k], a.p32[a.col[k]], s);
				a.w32[i] = s;
				q[0] = fma((double)s, (double)a.p32[i], q[0]);
			}
			team_sum<1>(q, sh_tree, slots, ph++, cl, team);
			const double alpha = rho / q[0];
			const float af = (float)alpha;
			// x32 += alpha p, r -= alpha w, ||r||^2, r . z
			double u[2] = {0.0, 0.0};
			for (int64_t i = r0 + tid; i < r1; i += nt) {
				a.x32[i] = fmaf(af, a.p32[i], a.x32[i]);
				const float ri = fmaf(-af, a.w32[i], a.r32[i]);
				a.r32[i] = ri;
				u[0] = fma((double)ri, (double)ri, u[0]);
				u[1] = fma((double)ri, (double)(a.dinv32[i] * ri), u[1]);
			}
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
			for (int64_t i = r0 + tid; i < r1; i += nt)
				a.p32[i] = fmaf(bf, a.p32[i], a.dinv32[i] * a.r32[i]);
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
};

// one plan per (matrix, partition); freed with the context process
std::map<std::pair<const Csr *, std::vector<int64_t>>, BatchPlan> g_plans;

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
	cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_cg, a);
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

	int cl = cluster_size, th = threads;
	if (cl == 0 || th == 0) {
		if (p.tuned_cluster == 0) {
			// autotuner, stage 1: time a short capped run of each cluster /
			// CTA size (every system a whole cluster) on this batch, keep the
			// fastest; the solution is restored afterwards
			std::vector<double> xsave(n);
			FS_CUDA_TRY(ctx, cudaMemcpy(xsave.data(), x->d, n * 8, cudaMemcpyDeviceToHost));
			BatchArgs t = a;
			t.maxiter = std::min(a.maxiter, 40);
			t.zero_guess = 1;
			float best = 1e30f;
			cudaEvent_t e0, e1;
			cudaEventCreate(&e0);
			cudaEventCreate(&e1);
			for (int c : {1, 2, 4, 8})
				for (int tt : {256, 512, 1024}) {
					if (cluster_size && c != cluster_size)
						continue;
					if (threads && tt != threads)
						continue;
					cudaEventRecord(e0, ctx->stream);
					int st = launch_batch(ctx, t, nsys, c, tt);
					cudaEventRecord(e1, ctx->stream);
					if (st != FS_OK) {
						cudaGetLastError();
						continue;
					}
					cudaEventSynchronize(e1);
					float ms = 0;
					cudaEventElapsedTime(&ms, e0, e1);
					if (ms < best) {
						best = ms;
						p.tuned_cluster = c;
						p.tuned_threads = tt;
					}
				}
			if (p.tuned_cluster == 0) {
				cudaEventDestroy(e0);
				cudaEventDestroy(e1);
				return set_err(ctx, FS_ERR_CUDA, "batched CG: no launch configuration ran");
			}
			// stage 2 (only when the caller fixed neither size): complete
			// solves -- capped runs cannot see that the largest systems also
			// need the most iterations -- of the stage-1 winner against
			// splits where the largest eighth or quarter of the systems own
			// a cluster of 4 or 8 CTAs and the rest one CTA each
			p.tuned_nbig = nsys;
			if (!cluster_size && !threads && nsys >= 8) {
				struct Cand { int c, t, nbig; };
				std::vector<Cand> cands = {{p.tuned_cluster, p.tuned_threads, nsys}};
				for (int c : {8, 4})
					for (int q : {8, 4})
						cands.push_back({c, 1024, std::max(1, nsys / q)});
				cands.push_back({8, 512, std::max(1, nsys / 4)});
				BatchArgs f = a;
				f.zero_guess = 1;
				float best2 = 1e30f;
				for (const Cand &cd : cands) {
					f.nbig = cd.nbig;
					cudaEventRecord(e0, ctx->stream);
					int st = launch_batch(ctx, f, nsys, cd.c, cd.t);
					cudaEventRecord(e1, ctx->stream);
					if (st != FS_OK) {
						cudaGetLastError();
						continue;
					}
					cudaEventSynchronize(e1);
					float ms = 0;
					cudaEventElapsedTime(&ms, e0, e1);
					if (ms < best2) {
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
