// Device Krylov loops: CG, BiCGSTAB, mixed-precision refined CG, and the
// solver object / C ABI shared with GMRES (gmres.cu).
//
// The loops follow the reference's control flow and scalar recurrences
// (flecsolve/solvers/cg.hh:43-139, bicgstab.hh:39-187); what changes is where
// the work runs.  Each reduction the reference performs with a host `.get()`
// (a FleCSI fold + MPI allreduce, vectors/operations/topo_view.hh:212-274)
// is fused into the kernel that produces its operands, and the kernel's last
// block finishes the scalar recurrence (alpha, beta, omega, convergence test)
// into a device-resident KState.  Nothing in an iteration needs the host, so
// k iterations are captured into one CUDA graph and the host reads the state
// back once per graph launch.  After convergence the remaining kernels of a
// graph return at their first instruction.
#include <cmath>
#include <cstring>
#include <type_traits>

#include "solver.cuh"

namespace fsg {

#define FOR_EACH(i, n)                                                          \
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n);  \
	     i += (int64_t)gridDim.x * blockDim.x)

constexpr int kThreads = 256;

__device__ __forceinline__ bool stopped(const KState *st) {
	return st->done || (st->flags & (KF_RESTART | KF_RELIABLE));
}

// ------------------------------------------------------ setup kernels --

// bnorm = ||b||, sol0 = ||x|| (when x is given); terminate_tol as cg.hh:55-62
// (CG/BiCGSTAB: b_norm == 0 -> 1) or gmres.hh:98-106 (b_norm < eps -> 1).
template<class V>
__global__ void __launch_bounds__(kThreads)
k_norms(int64_t n, const V *__restrict__ b, const V *__restrict__ x, KState *st,
        double *part, unsigned *counter, int gmres_rule) {
	__shared__ double sh[128];
	Acc<V, 2> acc;
	acc.init();
	FOR_EACH(i, n) {
		acc.add_prod(0, b[i], b[i]);
		if (x)
			acc.add_prod(1, x[i], x[i]);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[2];
		sum_partials<2>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			double bn = sqrt(s[0]);
			if (gmres_rule) {
				st->rhs_norm = bn;
				if (bn < 2.220446049250313e-16)
					bn = 1.0;
			}
			else {
				if (bn == 0.0)
					bn = 1.0;
				st->rhs_norm = bn;
			}
			st->bnorm = bn;
			st->tol = st->rtol * bn;
			st->sol0 = x ? sqrt(s[1]) : 0.0;
			*counter = 0;
		}
	}
}

template<class V>
__global__ void k_fill(int64_t n, V *__restrict__ x, V a) {
	FOR_EACH(i, n) x[i] = a;
}

template<class V>
__global__ void k_copy(int64_t n, const V *__restrict__ s, V *__restrict__ d) {
	FOR_EACH(i, n) d[i] = s[i];
}

__global__ void k_mul(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                      double *__restrict__ d) {
	FOR_EACH(i, n) d[i] = a[i] * b[i];
}

// ---------------------------------------------------------------- CG --

// z = P r (PK 0: identity, 1: diagonal); p = z; rho = z'r; res0 = ||r||
// (cg.hh:75-90).  Early exit when res0 < tol (cg.hh:77-82).
// The pending solution step of the reliable-update iteration starts at 0.
template<class V, int PK>
__global__ void __launch_bounds__(kThreads)
k_cg_start(int64_t n, const V *__restrict__ r, const V *__restrict__ dinv,
           V *__restrict__ p, KState *st, double *part, unsigned *counter) {
	__shared__ double sh[128];
	Acc<V, 2> acc;
	acc.init();
	FOR_EACH(i, n) {
		V ri = r[i];
		V zi = PK ? dinv[i] * ri : ri;
		p[i] = zi;
		acc.add_prod(0, ri, ri);
		acc.add_prod(1, zi, ri);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[2];
		sum_partials<2>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			double res = sqrt(s[0]);
			st->res0 = res;
			st->res = res;
			st->rho = s[1];
			st->rho_old = s[1];
			st->iter = 0;
			st->flags = 0;
			st->alpha_x = 0.0;
			if (res < st->tol) {
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
				st->info_iters = 0;
			}
			else if (st->maxiter <= 0) {
				st->done = 1;
				st->status = FS_DIVERGED_ITERS;
			}
			*counter = 0;
		}
	}
}

// w = A p and p'Ap -> alpha = rho / p'Ap (cg.hh:94-106)
template<class V>
struct EpiCgAp {
	static constexpr int NV = 1;
	V *w;
	const V *p;
	KState *st;
	double *part;
	unsigned *counter;
	__device__ bool skip() const { return stopped(st); }
	template<class A>
	__device__ void row(int r, V s, A &acc) const {
		w[r] = s;
		acc.add_prod(0, s, p[r]);
	}
	__device__ void finish(const double *s) const {
		double pap = s[0];
		st->pAp = pap;
		if (!(pap > 0.0))
			st->flags |= KF_NEG_CURVATURE;
		st->alpha = st->rho / pap;
	}
};

// x += alpha p; r -= alpha w; z = P r; ||r||, r'z; convergence test and
// beta = rho_new / rho_old (cg.hh:108-129)
template<class V, int PK>
__global__ void __launch_bounds__(kThreads)
k_cg_update(int64_t n, V *__restrict__ x, const V *__restrict__ p, V *__restrict__ r,
            const V *__restrict__ w, const V *__restrict__ dinv, KState *st,
            double *part, unsigned *counter, double *hist) {
	__shared__ double sh[128];
	pdl_wait();
	pdl_trigger();
	if (stopped(st))
		return;
	const V alpha = (V)st->alpha;
	Acc<V, 2> acc;
	acc.init();
	FOR_EACH(i, n) {
		V xi = fma(alpha, p[i], x[i]);
		V ri = fma(-alpha, w[i], r[i]);
		x[i] = xi;
		r[i] = ri;
		V zi = PK ? dinv[i] * ri : ri;
		acc.add_prod(0, ri, ri);
		acc.add_prod(1, ri, zi);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[2];
		sum_partials<2>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			double res = sqrt(s[0]);
			int it = st->iter + 1;
			st->iter = it;
			st->res = res;
			if (it <= st->hist_cap)
				hist[it - 1] = res;
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
				st->info_iters = 0;
			}
			st->rho_old = st->rho;
			st->rho = s[1];
			st->beta = s[1] / st->rho_old;
			*counter = 0;
		}
	}
}

// p = beta p + z, z = P r (cg.hh:124-130)
template<class V, int PK>
__global__ void __launch_bounds__(kThreads)
k_cg_dir(int64_t n, V *__restrict__ p, const V *__restrict__ r,
         const V *__restrict__ dinv, const KState *st) {
	pdl_wait();
	pdl_trigger();
	if (stopped(st))
		return;
	const V beta = (V)st->beta;
	FOR_EACH(i, n) {
		V zi = PK ? dinv[i] * r[i] : r[i];
		p[i] = fma(beta, p[i], zi);
	}
}

// -------------------------------------------------------- mixed (IR) --

// x64 += (double) d32 (refinement update)
__global__ void k_ir_update(int64_t n, double *__restrict__ x, const float *__restrict__ d) {
	FOR_EACH(i, n) x[i] += (double)d[i];
}

// r64 = b - A x (FP64), r32 = (float) r64, res = ||r64|| -> outer state
struct EpiIrResidual {
	static constexpr int NV = 1;
	const double *b;
	double *r64;
	float *r32;
	KState *st;
	double *part;
	unsigned *counter;
	__device__ bool skip() const { return false; }
	template<class A>
	__device__ void row(int r, double s, A &acc) const {
		double v = b[r] - s;
		r64[r] = v;
		r32[r] = (float)v;
		acc.add_prod(0, v, v);
	}
	__device__ void finish(const double *s) const {
		st->res = sqrt(s[0]);
		if (!isfinite(st->res))
			st->flags |= KF_NONFINITE;
	}
};

// inner solve set-up: tol_in = inner_rtol * ||r32||
__global__ void k_inner_init(KState *in, const KState *out, double inner_rtol, int maxiter) {
	in->tol = inner_rtol * out->res;
	in->rtol = inner_rtol;
	in->maxiter = maxiter;
	in->done = 0;
	in->status = FS_STATUS_UNKNOWN;
	in->iter = 0;
	in->flags = 0;
	in->info_iters = 0;
}

// Reliable-update variant (residual replacement, Sleijpen & van der Vorst
// 1996; van der Vorst & Ye 2000): the CG recurrences run in FP32 on a
// correction xs, and whenever the recurrence residual has dropped by `delta`
// since the last replacement (or below the tolerance) the host folds xs into
// the FP64 solution and replaces r by the FP64 true residual b - A x.  The
// search direction is kept, so no Krylov information is lost.  One iteration
// is three kernels: the SpMV with p'Ap, k_rc_resid4 (r -= alpha w, the dot
// products, the replacement test) and k_cg_dir_x (the solution step
// xs += alpha p and the direction update).

// x64 += xs; xs = 0
__global__ void k_rel_fold(int64_t n, double *__restrict__ x, float *__restrict__ xs) {
	FOR_EACH(i, n) {
		x[i] += (double)xs[i];
		xs[i] = 0.f;
	}
}

// ------------------------------------------- reliable-update CG loop --

// xs += alpha_x p (the pending solution step, cg.hh:108 in FP32); p = beta p
// + z, z = P r (cg.hh:124-130).  A replacement folds the pending step into x
// and clears alpha_x, so it is applied once.  Four elements per thread and
// pass (16-byte accesses; the solver's vectors and D^-1 are 16-byte aligned),
// the last n mod 4 elements one by one.
template<int PK>
__global__ void __launch_bounds__(kThreads)
k_cg_dir_x(int64_t n, float *__restrict__ p, const float *__restrict__ r,
           const float *__restrict__ dinv, float *__restrict__ xs, const KState *st) {
	pdl_wait();
	pdl_trigger();
	if (stopped(st))
		return;
	const float beta = (float)st->beta;
	const float ax = (float)st->alpha_x;
	auto one = [&](float &pi, float ri, float di, float &xi) {
		xi = fmaf(ax, pi, xi);
		pi = fmaf(beta, pi, PK ? di * ri : ri);
	};
	const int64_t n4 = n >> 2;
	float4 *p4 = reinterpret_cast<float4 *>(p), *x4 = reinterpret_cast<float4 *>(xs);
	const float4 *r4 = reinterpret_cast<const float4 *>(r);
	const float4 *d4 = reinterpret_cast<const float4 *>(dinv);
	FOR_EACH(i, n4) {
		float4 pv = p4[i], xv = x4[i];
		const float4 rv = r4[i];
		const float4 dv = PK ? __ldg(d4 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
		one(pv.x, rv.x, dv.x, xv.x);
		one(pv.y, rv.y, dv.y, xv.y);
		one(pv.z, rv.z, dv.z, xv.z);
		one(pv.w, rv.w, dv.w, xv.w);
		p4[i] = pv;
		x4[i] = xv;
	}
	for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x)
		one(p[i], r[i], PK ? dinv[i] : 0.f, xs[i]);
}

// r -= alpha w; z = P r; ||r||, r'z (cg.hh:109-123 in FP32, compensated
// sums); replacement test (the recurrence residual dropped by delta since the
// last replacement, or below the tolerance, or maxiter) and beta.  The
// solution step xs += alpha p of this iteration is left pending (alpha_x)
// for k_cg_dir_x, which reads p next.  Four elements per thread and pass.
template<int PK>
__global__ void __launch_bounds__(kThreads)
k_rc_resid4(int64_t n, float *__restrict__ r, const float *__restrict__ w,
            const float *__restrict__ dinv, KState *st, double *part, unsigned *counter,
            double *hist, double delta) {
	__shared__ double sh[128];
	pdl_wait();
	pdl_trigger();
	if (stopped(st))
		return;
	const float alpha = (float)st->alpha;
	Acc<float, 2> acc;
	acc.init();
	auto one = [&](float &ri, float wi, float di) {
		ri = fmaf(-alpha, wi, ri);
		const float zi = PK ? di * ri : ri;
		acc.add_prod(0, ri, ri);
		acc.add_prod(1, ri, zi);
	};
	const int64_t n4 = n >> 2;
	float4 *r4 = reinterpret_cast<float4 *>(r);
	const float4 *w4 = reinterpret_cast<const float4 *>(w);
	const float4 *d4 = reinterpret_cast<const float4 *>(dinv);
	FOR_EACH(i, n4) {
		float4 rv = r4[i];
		const float4 wv = w4[i];
		const float4 dv = PK ? __ldg(d4 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
		one(rv.x, wv.x, dv.x);
		one(rv.y, wv.y, dv.y);
		one(rv.z, wv.z, dv.z);
		one(rv.w, wv.w, dv.w);
		r4[i] = rv;
	}
	for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
	     i += (int64_t)gridDim.x * blockDim.x)
		one(r[i], w[i], PK ? dinv[i] : 0.f);
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[2];
		sum_partials<2>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			double res = sqrt(s[0]);
			int it = st->iter + 1;
			st->iter = it;
			st->res = res;
			if (it <= st->hist_cap)
				hist[it - 1] = res;
			if (!isfinite(res))
				st->flags |= KF_NONFINITE;
			if (res < delta * st->aux[1] || res < st->tol || it >= st->maxiter ||
			    (st->flags & KF_NONFINITE))
				st->flags |= KF_RELIABLE;
			st->rho_old = st->rho;
			st->rho = s[1];
			st->beta = s[1] / st->rho_old;
			st->alpha_x = st->alpha;
			*counter = 0;
		}
	}
}

// x64 += (xs + alpha_x p); xs = 0 -- the fold with the pending solution step
// of the last iteration
__global__ void k_rel_fold_pending(int64_t n, double *__restrict__ x, float *__restrict__ xs,
                                   const float *__restrict__ p, const KState *st) {
	const float a = (float)st->alpha_x;
	FOR_EACH(i, n) {
		x[i] += (double)fmaf(a, p[i], xs[i]);
		xs[i] = 0.f;
	}
}

// after the FP64 residual replaced r32: rho = r'Dr, beta = rho / rho_old,
// new reference level for the next replacement, stopping test
template<int PK>
__global__ void __launch_bounds__(kThreads)
k_rel_finish(int64_t n, const float *__restrict__ r, const float *__restrict__ dinv, KState *st,
             double *part, unsigned *counter) {
	__shared__ double sh[128];
	Acc<float, 1> acc;
	acc.init();
	FOR_EACH(i, n) {
		float ri = r[i];
		acc.add_prod(0, ri, PK ? dinv[i] * ri : ri);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[1];
		sum_partials<1>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			st->rho = s[0];
			st->beta = s[0] / st->rho_old;
			st->aux[1] = st->res;  // true residual after the replacement
			st->restarts += 1;     // number of replacements
			st->alpha_x = 0.0;     // the fold applied the pending step
			st->flags &= ~KF_RELIABLE;
			if (st->res < st->tol) {
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
				st->info_iters = st->iter;
			}
			else if (st->iter >= st->maxiter || (st->flags & KF_NONFINITE)) {
				st->done = 1;
				st->status = FS_DIVERGED_ITERS;
				st->info_iters = 0;
			}
			*counter = 0;
		}
	}
}

// The FP64 head of a reliable-update CG has reached its tolerance: the same
// Krylov process continues at the final tolerance with FP32 recurrences.
// After k >= 1 head iterations the next direction is z_k + beta_k p_{k-1}
// (beta_k from the replaced residual's rho over the head's last rho).  When
// the initial residual was already below the head's tolerance (k = 0, a
// warm start), the start kernel's p = z_0 is the first direction itself:
// beta must be 0 (rho_old = inf), or the direction would be scaled and the
// next ones would lose conjugacy.
__global__ void k_head_switch(KState *st, double rtol) {
	st->rtol = rtol;
	st->tol = rtol * st->bnorm;
	st->done = 0;
	st->status = FS_STATUS_UNKNOWN;
	st->info_iters = 0;
	st->flags = 0;
	st->alpha_x = 0.0;
	if (st->iter == 0)
		st->rho_old = INFINITY;
}

__global__ void k_to_f32(int64_t n, const double *__restrict__ s, float *__restrict__ d) {
	FOR_EACH(i, n) d[i] = (float)s[i];
}

// r64 = b - A x, r32 = (float) r64, st->res = ||r64|| (FP64)
struct EpiRelResidual {
	static constexpr int NV = 1;
	const double *b;
	float *r32;
	KState *st;
	double *part;
	unsigned *counter;
	__device__ bool skip() const { return false; }
	template<class A>
	__device__ void row(int r, double s, A &acc) const {
		double v = b[r] - s;
		r32[r] = (float)v;
		acc.add_prod(0, v, v);
	}
	__device__ void finish(const double *s) const {
		st->res = sqrt(s[0]);
		if (!isfinite(st->res))
			st->flags |= KF_NONFINITE;
	}
};

// --------------------------------------------------------- BiCGSTAB --

// res = b (zero guess) or b - A x done before; here: res_norm, r~ = res,
// p = v = 0, rho = r~'res (bicgstab.hh:73-98)
template<class V>
__global__ void __launch_bounds__(kThreads)
k_bi_start(int64_t n, const V *__restrict__ res, V *__restrict__ rt, V *__restrict__ p,
           V *__restrict__ v, KState *st, double *part, unsigned *counter) {
	__shared__ double sh[128];
	Acc<V, 1> acc;
	acc.init();
	FOR_EACH(i, n) {
		V ri = res[i];
		rt[i] = ri;
		p[i] = V(0);
		v[i] = V(0);
		acc.add_prod(0, ri, ri);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[1];
		sum_partials<1>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			double rn = sqrt(s[0]);
			st->res0 = rn;
			st->res = rn;
			st->r_tilde_norm = rn;
			st->alpha = 1.0;
			st->beta = 0.0;
			st->omega = 1.0;
			st->rho_old = 2.0;  // std::vector<real> rho{2, 1.0}
			st->rho = s[0];     // r~'res with r~ = res
			st->iter = 0;
			st->flags = 0;
			if (rn < st->tol) {
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
			}
			else if (st->maxiter <= 0) {
				st->done = 1;
				st->status = FS_DIVERGED_ITERS;
			}
			*counter = 0;
		}
	}
}

// p update (bicgstab.hh:115-122)
template<class V>
__global__ void k_bi_p(int64_t n, V *__restrict__ p, const V *__restrict__ v,
                       const V *__restrict__ res, const KState *st) {
	if (stopped(st))
		return;
	if (st->iter == 0) {
		FOR_EACH(i, n) p[i] = res[i];
	}
	else {
		const double bd = (st->rho / st->rho_old) * (st->alpha / st->omega);
		const V beta = (V)bd, om = (V)st->omega;
		auto one = [&](V &pi, V vi, V ri) { pi = fma(beta, fma(-om, vi, pi), ri); };
		if constexpr (std::is_same_v<V, float>) {
			// four elements a thread and pass (16-byte accesses; the solver's
			// FP32 vectors are 16-byte aligned), the last n mod 4 one by one
			const int64_t n4 = n >> 2;
			float4 *p4 = reinterpret_cast<float4 *>(p);
			const float4 *v4 = reinterpret_cast<const float4 *>(v);
			const float4 *r4 = reinterpret_cast<const float4 *>(res);
			FOR_EACH(i, n4) {
				float4 pv = p4[i];
				const float4 vv = v4[i], rv = r4[i];
				one(pv.x, vv.x, rv.x);
				one(pv.y, vv.y, rv.y);
				one(pv.z, vv.z, rv.z);
				one(pv.w, vv.w, rv.w);
				p4[i] = pv;
			}
			for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
			     i += (int64_t)gridDim.x * blockDim.x)
				one(p[i], v[i], res[i]);
		}
		else {
			FOR_EACH(i, n) one(p[i], v[i], res[i]);
		}
	}
}

// v = A P p, alpha = rho / r~'v (bicgstab.hh:124-130)
template<class V>
struct EpiBiV {
	static constexpr int NV = 1;
	V *v;
	const V *rt;
	KState *st;
	double *part;
	unsigned *counter;
	__device__ bool skip() const { return stopped(st); }
	template<class A>
	__device__ void row(int r, V s, A &acc) const {
		v[r] = s;
		acc.add_prod(0, rt[r], s);
	}
	__device__ void finish(const double *s) const {
		if (!(s[0] != 0.0)) {
			st->flags |= KF_ALPHA_ZERO;
			st->done = 1;
			st->status = FS_DIVERGED_BREAKDOWN;
			return;
		}
		st->alpha = st->rho / s[0];
	}
};

// s = res - alpha v, s_norm; early exit when s_norm < rtol (bicgstab.hh:132-143)
template<class V>
__global__ void __launch_bounds__(kThreads)
k_bi_s(int64_t n, V *__restrict__ s, const V *__restrict__ v, const V *__restrict__ res,
       KState *st, double *part, unsigned *counter) {
	__shared__ double sh[128];
	if (stopped(st))
		return;
	const V a = (V)st->alpha;
	Acc<V, 1> acc;
	acc.init();
	auto one = [&](V &si, V vi, V ri) {
		si = fma(-a, vi, ri);
		acc.add_prod(0, si, si);
	};
	if constexpr (std::is_same_v<V, float>) {
		// four elements a thread and pass, as k_bi_p
		const int64_t n4 = n >> 2;
		float4 *s4 = reinterpret_cast<float4 *>(s);
		const float4 *v4 = reinterpret_cast<const float4 *>(v);
		const float4 *r4 = reinterpret_cast<const float4 *>(res);
		FOR_EACH(i, n4) {
			float4 sv;
			const float4 vv = v4[i], rv = r4[i];
			one(sv.x, vv.x, rv.x);
			one(sv.y, vv.y, rv.y);
			one(sv.z, vv.z, rv.z);
			one(sv.w, vv.w, rv.w);
			s4[i] = sv;
		}
		for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
		     i += (int64_t)gridDim.x * blockDim.x)
			one(s[i], v[i], res[i]);
	}
	else {
		FOR_EACH(i, n) one(s[i], v[i], res[i]);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double sum[1];
		sum_partials<1>(part, gridDim.x, sum, sh);
		if (threadIdx.x == 0) {
			double sn = sqrt(sum[0]);
			st->s_norm = sn;
			if (sn < st->rtol)
				st->flags |= KF_EARLY;
			*counter = 0;
		}
	}
}

// t = A P s, t't, t's -> omega (bicgstab.hh:145-151)
template<class V>
struct EpiBiT {
	static constexpr int NV = 2;
	V *t;
	const V *s;
	KState *st;
	double *part;
	unsigned *counter;
	__device__ bool skip() const { return stopped(st) || (st->flags & KF_EARLY); }
	template<class A>
	__device__ void row(int r, V val, A &acc) const {
		t[r] = val;
		acc.add_prod(0, val, val);
		acc.add_prod(1, val, s[r]);
	}
	__device__ void finish(const double *q) const {
		st->t_sq = q[0];
		st->t_s = q[1];
		st->omega = (q[0] == 0.0) ? 0.0 : q[1] / q[0];
	}
};

// x += alpha P p (+ omega P s); res = s - omega t; ||res||, r~'res; tests
// (bicgstab.hh:136-178, with the next iteration's rho = r~'res fused in)
//
// RELY (mixed precision): the FP32 recurrence never stops by itself; every
// stop condition, and a residual drop by aux[0] since the last replacement,
// raises KF_RELIABLE with the reason in aux[3] (0 drop, 1 converged, 2 early
// exit, 3 omega == 0, 4 maxiter) and the host replaces the residual by the
// FP64 one before deciding.
template<class V, int PK, bool RELY = false>
__global__ void __launch_bounds__(kThreads)
k_bi_x(int64_t n, V *__restrict__ x, const V *__restrict__ p, const V *__restrict__ s,
       const V *__restrict__ t, V *__restrict__ res, const V *__restrict__ rt,
       const V *__restrict__ dinv, KState *st, double *part, unsigned *counter,
       double *hist) {
	__shared__ double sh[128];
	if (stopped(st))
		return;
	const V a = (V)st->alpha;
	if (st->flags & KF_EARLY) {
		FOR_EACH(i, n) {
			V ph = PK ? dinv[i] * p[i] : p[i];
			x[i] = fma(a, ph, x[i]);
		}
		// the state changes only once every block has passed its entry test
		if (last_block(counter) && threadIdx.x == 0) {
			if (RELY) {
				st->flags |= KF_RELIABLE;
				st->aux[3] = 2;
			}
			else {
				st->info_iters = st->iter;
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
			}
			*counter = 0;
		}
		return;
	}
	const V om = (V)st->omega;
	Acc<V, 2> acc;
	acc.init();
	auto one = [&](V &xi, V &ri, V pi, V si, V ti, V rti, V di) {
		const V ph = PK ? di * pi : pi;
		const V sh_ = PK ? di * si : si;
		xi = fma(om, sh_, fma(a, ph, xi));
		ri = fma(-om, ti, si);
		acc.add_prod(0, ri, ri);
		acc.add_prod(1, rti, ri);
	};
	if constexpr (std::is_same_v<V, float>) {
		// four elements a thread and pass, as k_bi_p
		const int64_t n4 = n >> 2;
		float4 *x4 = reinterpret_cast<float4 *>(x), *r4 = reinterpret_cast<float4 *>(res);
		const float4 *p4 = reinterpret_cast<const float4 *>(p);
		const float4 *s4 = reinterpret_cast<const float4 *>(s);
		const float4 *t4 = reinterpret_cast<const float4 *>(t);
		const float4 *q4 = reinterpret_cast<const float4 *>(rt);
		const float4 *d4 = reinterpret_cast<const float4 *>(dinv);
		FOR_EACH(i, n4) {
			float4 xv = x4[i], rv;
			const float4 pv = p4[i], sv = s4[i], tv = t4[i], qv = q4[i];
			const float4 dv = PK ? d4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
			one(xv.x, rv.x, pv.x, sv.x, tv.x, qv.x, dv.x);
			one(xv.y, rv.y, pv.y, sv.y, tv.y, qv.y, dv.y);
			one(xv.z, rv.z, pv.z, sv.z, tv.z, qv.z, dv.z);
			one(xv.w, rv.w, pv.w, sv.w, tv.w, qv.w, dv.w);
			x4[i] = xv;
			r4[i] = rv;
		}
		for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
		     i += (int64_t)gridDim.x * blockDim.x)
			one(x[i], res[i], p[i], s[i], t[i], rt[i], PK ? dinv[i] : 0.f);
	}
	else {
		FOR_EACH(i, n) one(x[i], res[i], p[i], s[i], t[i], rt[i], PK ? dinv[i] : V(0));
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double q[2];
		sum_partials<2>(part, gridDim.x, q, sh);
		if (threadIdx.x == 0) {
			double rn = sqrt(q[0]);
			int it = st->iter;
			st->res = rn;
			const int hi = st->nhist;
			if (hi < st->hist_cap)
				hist[hi] = rn;
			st->nhist = hi + 1;
			if (!isfinite(rn))
				st->flags |= KF_NONFINITE;
			if (RELY) {
				int why = -1;
				if (rn < st->tol)
					why = 1;
				else if (st->omega == 0.0)
					why = 3;
				else if (it + 1 >= st->maxiter || (st->flags & KF_NONFINITE))
					why = 4;
				else if (rn < st->aux[0] * st->aux[1])
					why = 0;
				if (why >= 0) {
					st->flags |= KF_RELIABLE;
					st->aux[3] = why;
				}
			}
			else if (rn < st->tol) {
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
				st->info_iters = it + 1;
			}
			else if (st->omega == 0.0) {
				st->done = 1;
				st->status = FS_DIVERGED_BREAKDOWN;
				st->info_iters = it + 1;
			}
			st->rho_old = st->rho;
			st->rho = q[1];
			st->iter = it + 1;
			if (!st->done && !(st->flags & KF_RELIABLE)) {
				if (it + 1 >= st->maxiter || (st->flags & KF_NONFINITE)) {
					st->done = 1;
					st->status = FS_DIVERGED_ITERS;
				}
				else if (sqrt(fabs(q[1])) < 2.220446049250313e-16 * st->r_tilde_norm) {
					st->flags |= KF_RESTART;
				}
			}
			*counter = 0;
		}
	}
}

// mixed BiCGSTAB: decision after the FP64 residual replaced res (st->res)
__global__ void k_bi_rel_decide(KState *st) {
	const int why = (int)st->aux[3];
	st->flags &= ~(KF_RELIABLE | KF_EARLY);
	st->aux[3] = 0;
	if (st->res < st->tol) {
		st->done = 1;
		st->status = FS_CONVERGED_RTOL;
		st->info_iters = st->iter;
	}
	else if (why == 3) {
		st->done = 1;
		st->status = FS_DIVERGED_BREAKDOWN;
		st->info_iters = st->iter;
	}
	else if (why == 4 || st->iter >= st->maxiter || (st->flags & KF_NONFINITE)) {
		st->done = 1;
		st->status = FS_DIVERGED_ITERS;
	}
	else {
		st->aux[1] = st->res;
		if (why == 2 || why == 1)
			st->flags |= KF_RESTART;  // the recurrence is spent: restart from r
	}
}

// rho = r~ . res after a replacement (the next iteration's rho_1)
template<class V>
__global__ void __launch_bounds__(kThreads)
k_bi_rho(int64_t n, const V *__restrict__ rt, const V *__restrict__ res, KState *st,
         double *part, unsigned *counter) {
	__shared__ double sh[128];
	if (st->done || (st->flags & KF_RESTART))
		return;
	Acc<V, 1> acc;
	acc.init();
	FOR_EACH(i, n) acc.add_prod(0, rt[i], res[i]);
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double q[1];
		sum_partials<1>(part, gridDim.x, q, sh);
		if (threadIdx.x == 0) {
			st->rho = q[0];
			*counter = 0;
		}
	}
}

// restart set-up after the host recomputed res = b - A x (bicgstab.hh:106-112):
// r~ = res, p = res, r_tilde_norm = ||res||, rho = r~'res for the next pass
template<class V>
__global__ void __launch_bounds__(kThreads)
k_bi_restart(int64_t n, const V *__restrict__ res, V *__restrict__ rt, V *__restrict__ p,
             KState *st, double *part, unsigned *counter) {
	__shared__ double sh[128];
	Acc<V, 1> acc;
	acc.init();
	FOR_EACH(i, n) {
		V ri = res[i];
		rt[i] = ri;
		p[i] = ri;
		acc.add_prod(0, ri, ri);
	}
	acc.to_part(part, sh);
	if (last_block(counter)) {
		double s[1];
		sum_partials<1>(part, gridDim.x, s, sh);
		if (threadIdx.x == 0) {
			double rn = sqrt(s[0]);
			st->res = rn;
			st->r_tilde_norm = rn;
			st->rho = s[0];  // recomputed r~'res of the next iteration
			st->restarts += 1;
			st->flags &= ~KF_RESTART;
			// the reference's restart `continue`s: it consumes a loop index
			st->iter += 1;
			if (st->iter >= st->maxiter) {
				st->done = 1;
				st->status = FS_DIVERGED_ITERS;
			}
			*counter = 0;
		}
	}
}

// ------------------------------------------------------- solver core --

const double *Solver::dinv64() const {
	if (P.kind == FS_PRECOND_JACOBI)
		return A->dinv;
	if (P.kind == FS_PRECOND_DIAG)
		return (const double *)w64[10];
	return nullptr;
}
const float *Solver::dinv32() const {
	if (P.kind == FS_PRECOND_JACOBI)
		return A->dinv32;
	if (P.kind == FS_PRECOND_DIAG)
		return w32[10];
	return nullptr;
}

static int dalloc(Solver *s, void **p, size_t bytes) {
	cudaError_t e = cudaMalloc(p, bytes);
	if (e != cudaSuccess) {
		cudaGetLastError();
		return set_err(s->ctx, FS_ERR_OUT_OF_MEMORY, "solver work allocation of %zu bytes failed",
		               bytes);
	}
	s->bufs.push_back(*p);
	return cudaMemsetAsync(*p, 0, bytes, s->ctx->stream) == cudaSuccess ? FS_OK : FS_ERR_CUDA;
}

int solver_alloc(Solver *s) {
	if (s->st)
		return FS_OK;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const size_t n64 = (size_t)((n + 31) / 32 * 32 + 32) * 8;
	const size_t n32 = (size_t)((n + 31) / 32 * 32 + 32) * 4;
	int nw64 = 0, nw32 = 0;
	switch (s->method) {
	case FS_CG: nw64 = 3; break;
	case FS_BICGSTAB: nw64 = 6; break;
	case FS_GMRES: nw64 = 3; break;
	case FS_CG_MIXED: nw64 = 1; nw32 = 5; break;
	case FS_CG_PIPELINED: nw64 = 5; break;
	case FS_BICGSTAB_MIXED: nw64 = 1; nw32 = 7; break;
	case FS_GMRES_MIXED: nw64 = 3; nw32 = 3; break;
	}
	for (int i = 0; i < nw64; ++i)
		FS_TRY(dalloc(s, (void **)&s->w64[i], n64));
	for (int i = 0; i < nw32; ++i)
		FS_TRY(dalloc(s, (void **)&s->w32[i], n32));
	FS_TRY(dalloc(s, (void **)&s->st, sizeof(KState)));
	FS_TRY(dalloc(s, (void **)&s->st_in, sizeof(KState)));
	// reduction partials: up to 8 CTAs per SM, up to 32 values per CTA (the
	// GMRES multi-dot of gmres.cu); every kernel's grid is <= 8 * SMs
	FS_TRY(dalloc(s, (void **)&s->part, sizeof(double) * (size_t)ctx->sms * 8 * kPartPerBlock + 1024));
	FS_TRY(dalloc(s, (void **)&s->counter, 64));
	const bool gm = s->method == FS_GMRES || s->method == FS_GMRES_MIXED;
	FS_TRY(dalloc(s, (void **)&s->hdev, gm ? sizeof(GmState) : sizeof(double) * 4096));
	cudaError_t e = cudaMallocHost(&s->hst, sizeof(KState));
	if (e != cudaSuccess)
		return set_err(ctx, FS_ERR_OUT_OF_MEMORY, "pinned state allocation failed");
	memset(s->hst, 0, sizeof(KState));
	if (s->P.kind == FS_PRECOND_DIAG) {
		// keep an FP64 and an FP32 copy of the caller's diagonal
		FS_TRY(dalloc(s, (void **)&s->w64[10], n64));
		FS_TRY(dalloc(s, (void **)&s->w32[10], n32));
	}
	if (s->P.kind == FS_PRECOND_JACOBI)
		FS_TRY(ensure_dinv(s->A));
	const bool mixed =
		s->method == FS_CG_MIXED || s->method == FS_BICGSTAB_MIXED || s->method == FS_GMRES_MIXED;
	if (mixed)
		FS_TRY(ensure_val32(s->A));
	// choose the column-id SpMV schedule now, outside any graph capture
	if (!stores_no_rows(s->A)) {
		spmv_lanes(ctx, s->A, false);
		if (mixed)
			spmv_lanes(ctx, s->A, true);
	}
	return FS_OK;
}

int solver_hist(Solver *s, int cap) {
	if (cap <= s->hist_cap && s->hist)
		return FS_OK;
	if (s->hist)
		cudaFree(s->hist);
	s->hist = nullptr;
	FS_CUDA_TRY(s->ctx, cudaMalloc(&s->hist, sizeof(double) * (size_t)(cap + 1)));
	s->hist_cap = cap;
	return FS_OK;
}

int read_state(Solver *s) {
	FS_CUDA_TRY(s->ctx, cudaMemcpyAsync(s->hst, s->st, sizeof(KState), cudaMemcpyDeviceToHost,
	                                    s->ctx->stream));
	return check_device_error(s->ctx);  // synchronises the stream
}

// Capture `body` (k iterations) once per key, then replay it.
int graph_run(Solver *s, const GraphKey &key_in, int (*body)(Solver *, void *), void *arg) {
	Ctx *ctx = s->ctx;
	// a graph embeds the SpMV kernels chosen at capture: the formats in use
	// are part of the key, so a format that changes with the values (the
	// symmetric storage) or by request gets its own capture
	GraphKey key = key_in;
	key.fmt = active_coding(s->A, false) * 8 + active_coding(s->A, true) +
	          16 * (s->A->vec_lanes[0] + 1) + 1024 * (s->A->vec_lanes[1] + 1);
	const auto gkey = std::make_pair((const Csr *)s->A, key);
	auto it = s->graphs.find(gkey);
	if (it == s->graphs.end()) {
		int64_t before = ctx->launches;
		FS_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
		int st = body(s, arg);
		cudaGraph_t g = nullptr;
		cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
		int nodes = (int)(ctx->launches - before);
		ctx->launches = before;
		if (st != FS_OK) {
			if (g)
				cudaGraphDestroy(g);
			return st;
		}
		if (e != cudaSuccess)
			return set_err(ctx, FS_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
		cudaGraphExec_t ge = nullptr;
		e = cudaGraphInstantiate(&ge, g, 0);
		cudaGraphDestroy(g);
		if (e != cudaSuccess)
			return set_err(ctx, FS_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
		if (s->graphs.size() >= Solver::kMaxGraphs) {
			// evict the least recently launched graph once the stream has
			// drained (it may be the one still running)
			auto lru = s->graphs.begin();
			for (auto jt = s->graphs.begin(); jt != s->graphs.end(); ++jt)
				if (jt->second.last_use < lru->second.last_use)
					lru = jt;
			FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
			cudaGraphExecDestroy(lru->second.exec);
			s->graphs.erase(lru);
		}
		it = s->graphs.emplace(gkey, Solver::GraphEntry{ge, nodes, 0}).first;
	}
	it->second.last_use = ++s->graph_tick;
	FS_CUDA_TRY(ctx, cudaGraphLaunch(it->second.exec, ctx->stream));
	ctx->launches += it->second.nodes;
	return FS_OK;
}

static void clear_graphs(Solver *s) {
	for (auto &kv : s->graphs)
		cudaGraphExecDestroy(kv.second.exec);
	s->graphs.clear();
}

// Iterations per graph launch.  A launch records k iterations; those after
// convergence still launch their kernels, which return at once.  So a solve
// starts with short launches and doubles them while it runs, up to the
// configured count: a solve that converges in a few iterations (an inner or
// time-step solve) launches few idle iterations, and a long one soon runs at
// full length.  After a restart of the recurrences the next launch is sized
// to the length of the segment that just ended.
struct Chunk {
	static constexpr int kFirst = 4;
	int kmax, k;
	explicit Chunk(int kmax_) : kmax(kmax_), k(std::min(kFirst, kmax_)) {}
	void grow() { k = std::min(kmax, 2 * k); }
	void restart(int64_t segment) {
		int c = kFirst;
		while (c < segment && c < kmax)
			c *= 2;
		k = std::min(c, kmax);
	}
};

// Common loop driver: launch the captured k-iteration body until the device
// says done; call the user diagnostic for every new history entry.  `*k` is
// the iteration count the body records, `code` + 2 k its graph key.
struct LoopSpec {
	Vec *x;
	GraphKey key;
	int (*body)(Solver *, void *);
	void *arg;
	int (*on_restart)(Solver *, void *);  // BiCGSTAB restart handler
	int *k;
	int code;
};

static int run_loop(Solver *s, const LoopSpec &L, int *user_stop) {
	*user_stop = 0;
	int64_t seen = 0;
	Chunk chunk(*L.k);
	for (;;) {
		*L.k = chunk.k;
		GraphKey key = L.key;
		key.k = L.code + 2 * chunk.k;
		FS_TRY(graph_run(s, key, L.body, L.arg));
		chunk.grow();
		FS_TRY(read_state(s));
		KState &h = *s->hst;
		int64_t nh = s->method == FS_BICGSTAB ? (int64_t)h.nhist : h.iter;
		if (s->diag && nh > seen) {
			int64_t upto = std::min<int64_t>(nh, s->hist_cap);
			std::vector<double> hh(upto - seen > 0 ? upto - seen : 0);
			if (!hh.empty())
				FS_CUDA_TRY(s->ctx, cudaMemcpy(hh.data(), s->hist + seen, hh.size() * sizeof(double),
				                               cudaMemcpyDeviceToHost));
			for (size_t j = 0; j < hh.size(); ++j) {
				if (s->diag(s->diag_user, reinterpret_cast<fs_vec>(L.x), hh[j])) {
					*user_stop = (int)(seen + j + 1);
					return FS_OK;
				}
			}
			seen = nh;
		}
		else {
			seen = nh;
		}
		if (h.done)
			return FS_OK;
		if ((h.flags & KF_RESTART) && L.on_restart)
			FS_TRY(L.on_restart(s, L.arg));
	}
}

// ---------------------------------------------------- CG apply (FP64) --

struct CgArgs {
	Vec *b, *x;
	int k;
};

template<int PK>
static int cg_body64(Solver *s, void *a) {
	CgArgs *g = (CgArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	double *r = s->w64[0], *p = s->w64[1], *w = s->w64[2];
	double *x = (double *)g->x->d;
	const double *dinv = s->dinv64();
	const int G = red_grid(ctx, n);
	for (int k = 0; k < g->k; ++k) {
		FS_TRY(launch_spmv<double, false, false>(
			ctx, s->A, s->A->val, p, nullptr,
			EpiCgAp<double>{w, p, s->st, s->part, s->counter}));
		FS_TRY(check_launch_rc(ctx,
		                       launch_pdl(ctx->stream, k_cg_update<double, PK>, G, kThreads, 0, n, x, p,
		                                  r, w, dinv, s->st, s->part, s->counter, s->hist),
		                       "cg update"));
		FS_TRY(check_launch_rc(ctx, launch_pdl(ctx->stream, k_cg_dir<double, PK>, G, kThreads, 0, n, p, r,
		                                       dinv, (const KState *)s->st),
		                       "cg direction"));
	}
	return FS_OK;
}

template<int PK>
static int cg_body32(Solver *s, void *a) {
	CgArgs *g = (CgArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	float *r = s->w32[0], *p = s->w32[1], *w = s->w32[2], *x = s->w32[3];
	const float *dinv = s->dinv32();
	const int G = red_grid(ctx, n);
	for (int k = 0; k < g->k; ++k) {
		FS_TRY(launch_spmv<float, false, false>(
			ctx, s->A, s->A->val32, p, nullptr,
			EpiCgAp<float>{w, p, s->st_in, s->part, s->counter}));
		FS_TRY(check_launch_rc(ctx,
		                       launch_pdl(ctx->stream, k_cg_update<float, PK>, G, kThreads, 0, n, x, p, r,
		                                  w, dinv, s->st_in, s->part, s->counter, s->hist),
		                       "cg update f32"));
		FS_TRY(check_launch_rc(ctx, launch_pdl(ctx->stream, k_cg_dir<float, PK>, G, kThreads, 0, n, p, r,
		                                       dinv, (const KState *)s->st_in),
		                       "cg direction f32"));
	}
	return FS_OK;
}

static int init_state(Solver *s, KState *dst, double rtol, int maxiter) {
	KState h{};
	h.rtol = rtol;
	h.maxiter = maxiter;
	h.status = FS_STATUS_UNKNOWN;
	h.hist_cap = s->hist_cap;
	FS_CUDA_TRY(s->ctx, cudaMemcpyAsync(dst, &h, sizeof(KState), cudaMemcpyHostToDevice, s->ctx->stream));
	// the pageable source is consumed before the call returns
	return FS_OK;
}

int solver_norms(Solver *s, Vec *b, Vec *x, bool with_x, int gmres_rule) {
	Ctx *ctx = s->ctx;
	const int G = red_grid(ctx, s->n);
	k_norms<double><<<G, kThreads, 0, ctx->stream>>>(s->n, (const double *)b->d,
	                                                 with_x ? (const double *)x->d : nullptr,
	                                                 s->st, s->part, s->counter, gmres_rule);
	return check_launch(ctx, "norms");
}

static int sol_norm(Solver *s, Vec *x, double *out) {
	return fs_vec_l2norm(reinterpret_cast<fs_vec>(x), out);
}

static int k_default(const Solver *s) {
	int k = s->set.k_readback;
	if (k <= 0)
		k = 32;
	if (s->diag)
		k = 1;
	return k;
}

static int cg_apply64(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const int G = red_grid(ctx, n);
	const bool zg = s->set.base.use_zero_guess != 0;
	const int PK = s->dinv64() ? 1 : 0;
	double *r = s->w64[0], *p = s->w64[1];
	FS_TRY(solver_hist(s, std::max(1, s->set.base.maxiter)));
	FS_TRY(init_state(s, s->st, (double)s->set.base.rtol, s->set.base.maxiter));
	FS_TRY(solver_norms(s, b, x, !zg, 0));
	if (zg) {
		k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
		FS_TRY(check_launch(ctx, "fill"));
		k_copy<double><<<G, kThreads, 0, ctx->stream>>>(n, (const double *)b->d, r);
		FS_TRY(check_launch(ctx, "copy"));
	}
	else {
		FS_TRY(launch_spmv<double, false, false>(ctx, s->A, s->A->val, (const double *)x->d, nullptr,
		                                         EpiResidual<double>{(const double *)b->d, r}));
	}
	if (PK)
		k_cg_start<double, 1><<<G, kThreads, 0, ctx->stream>>>(n, r, s->dinv64(), p, s->st, s->part, s->counter);
	else
		k_cg_start<double, 0><<<G, kThreads, 0, ctx->stream>>>(n, r, nullptr, p, s->st, s->part, s->counter);
	FS_TRY(check_launch(ctx, "cg start"));
	FS_TRY(read_state(s));
	int user_stop = 0;
	if (!s->hst->done) {
		CgArgs args{b, x, k_default(s)};
		LoopSpec L{x, {b->d, x->d, 0}, PK ? cg_body64<1> : cg_body64<0>, &args, nullptr, &args.k, PK};
		FS_TRY(run_loop(s, L, &user_stop));
	}
	KState &h = *s->hst;
	s->hhist_count = std::min<int64_t>(h.iter, s->hist_cap);
	double xn = 0;
	FS_TRY(sol_norm(s, x, &xn));
	memset(info, 0, sizeof(*info));
	info->rhs_norm = (float)h.rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)h.sol0;
	info->res_norm_initial = (float)h.res0;
	info->sol_norm_final = (float)xn;
	info->res_norm_final = (float)h.res;
	if (user_stop) {
		info->status = FS_CONVERGED_USER;
		info->iters = user_stop;
	}
	else {
		info->status = h.status;
		info->iters = h.info_iters;
		if (h.iter > 0 && info->iters == 0)
			info->status = FS_DIVERGED_ITERS;  // cg.hh:135-136
	}
	if (h.flags & KF_NONFINITE)
		return set_err(ctx, FS_ERR_NON_FINITE, "CG: non-finite residual norm");
	return FS_OK;
}

// ---------------------------------- single-reduction (pipelined) CG --
//
// Chronopoulos & Gear (1989): the CG recurrences of cg.hh:43-139 rearranged
// so that an iteration has ONE grid-wide reduction.  With u = P r and w = A u
// carried along, the two dots gamma = (r, u) and delta = (w, u) (and the
// stopping norm ||r||) are all available right after the SpMV w = A u, so they
// are summed in that kernel's epilogue; the other kernel applies every vector
// update at once:
//   p = u + beta p,  s = w + beta s,  x += alpha p,  r -= alpha s,  u = P r
//   w = A u;  gamma' = (r, u), delta = (w, u), ||r||
//   beta = gamma' / gamma,  alpha = gamma' / (delta - beta gamma' / alpha)
// Two kernels and one reduction per iteration instead of three and two, at
// the price of two more vectors (s, w) streamed: 12 vector accesses in the
// update instead of 11 over the update and the direction kernels.  The
// stopping test is the reference's, on ||r|| after the update.

// p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s, u = P r
template<int PK>
__global__ void __launch_bounds__(kThreads)
k_pcg_update(int64_t n, double *__restrict__ x, double *__restrict__ r, double *__restrict__ u,
             const double *__restrict__ w, double *__restrict__ p, double *__restrict__ s,
             const double *__restrict__ dinv, const KState *st) {
	pdl_wait();
	pdl_trigger();
	if (stopped(st))
		return;
	const double alpha = st->alpha, beta = st->beta;
	FOR_EACH(i, n) {
		const double pi = fma(beta, p[i], u[i]);
		const double si = fma(beta, s[i], w[i]);
		x[i] = fma(alpha, pi, x[i]);
		const double ri = fma(-alpha, si, r[i]);
		p[i] = pi;
		s[i] = si;
		r[i] = ri;
		u[i] = PK ? dinv[i] * ri : ri;
	}
}

// w = A u and the iteration's three dots; the last CTA counts the iteration,
// tests ||r|| and forms beta, alpha (the first call, iter < 0: the start)
struct EpiPipe {
	static constexpr int NV = 3;
	double *w;
	const double *u, *r;
	KState *st;
	double *part;
	unsigned *counter;
	double *hist;
	__device__ bool skip() const { return stopped(st); }
	template<class A>
	__device__ void row(int i, double s, A &acc) const {
		w[i] = s;
		const double ui = u[i], ri = r[i];
		acc.add_prod(0, ri, ui);
		acc.add_prod(1, s, ui);
		acc.add_prod(2, ri, ri);
	}
	__device__ void finish(const double *sm) const {
		const double gamma = sm[0], delta = sm[1];
		const double res = sqrt(sm[2]);
		if (st->aux[0] == 0.0) {
			// the start (cg.hh:75-90): alpha = gamma / delta, beta = 0
			st->aux[0] = 1.0;
			st->res0 = res;
			st->res = res;
			st->rho = gamma;
			st->beta = 0.0;
			st->alpha = gamma / delta;
			if (res < st->tol) {
				st->done = 1;
				st->status = FS_CONVERGED_RTOL;
				st->info_iters = 0;
			}
			else if (st->maxiter <= 0) {
				st->done = 1;
				st->status = FS_DIVERGED_ITERS;
			}
			return;
		}
		const int it = st->iter + 1;
		st->iter = it;
		st->res = res;
		if (it <= st->hist_cap)
			hist[it - 1] = res;
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
			st->info_iters = 0;
		}
		const double beta = gamma / st->rho;
		st->beta = beta;
		st->alpha = gamma / (delta - beta * gamma / st->alpha);
		st->rho = gamma;
	}
};

template<int PK>
static int pcg_body(Solver *s, void *a) {
	CgArgs *g = (CgArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	double *r = s->w64[0], *u = s->w64[1], *w = s->w64[2], *p = s->w64[3], *sv = s->w64[4];
	double *x = (double *)g->x->d;
	const double *dinv = s->dinv64();
	const int G = red_grid(ctx, n);
	for (int k = 0; k < g->k; ++k) {
		FS_TRY(check_launch_rc(ctx,
		                       launch_pdl(ctx->stream, k_pcg_update<PK>, G, kThreads, 0, n, x, r, u,
		                                  (const double *)w, p, sv, dinv, (const KState *)s->st),
		                       "pipelined cg update"));
		FS_TRY(launch_spmv<double, false, false>(
			ctx, s->A, s->A->val, u, nullptr,
			EpiPipe{w, u, r, s->st, s->part, s->counter, s->hist}));
	}
	return FS_OK;
}

static int cg_apply_pipelined(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const int G = red_grid(ctx, n);
	const bool zg = s->set.base.use_zero_guess != 0;
	const int PK = s->dinv64() ? 1 : 0;
	double *r = s->w64[0], *u = s->w64[1], *w = s->w64[2], *p = s->w64[3], *sv = s->w64[4];
	FS_TRY(solver_hist(s, std::max(1, s->set.base.maxiter)));
	FS_TRY(init_state(s, s->st, (double)s->set.base.rtol, s->set.base.maxiter));
	FS_TRY(solver_norms(s, b, x, !zg, 0));
	if (zg) {
		k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
		FS_TRY(check_launch(ctx, "fill"));
		k_copy<double><<<G, kThreads, 0, ctx->stream>>>(n, (const double *)b->d, r);
		FS_TRY(check_launch(ctx, "copy"));
	}
	else {
		FS_TRY(launch_spmv<double, false, false>(ctx, s->A, s->A->val, (const double *)x->d, nullptr,
		                                         EpiResidual<double>{(const double *)b->d, r}));
	}
	// u = P r, p = s = 0, then w = A u with the start's dots
	if (PK)
		k_mul<<<G, kThreads, 0, ctx->stream>>>(n, s->dinv64(), r, u);
	else
		k_copy<double><<<G, kThreads, 0, ctx->stream>>>(n, r, u);
	FS_TRY(check_launch(ctx, "pipelined cg start"));
	k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, p, 0.0);
	k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, sv, 0.0);
	FS_TRY(check_launch(ctx, "fill"));
	FS_TRY(launch_spmv<double, false, false>(ctx, s->A, s->A->val, u, nullptr,
	                                         EpiPipe{w, u, r, s->st, s->part, s->counter, s->hist}));
	FS_TRY(read_state(s));
	int user_stop = 0;
	if (!s->hst->done) {
		CgArgs args{b, x, k_default(s)};
		LoopSpec L{x, {b->d, x->d, 0}, PK ? pcg_body<1> : pcg_body<0>, &args, nullptr, &args.k,
		           6000 + PK};
		FS_TRY(run_loop(s, L, &user_stop));
	}
	KState &h = *s->hst;
	s->hhist_count = std::min<int64_t>(h.iter, s->hist_cap);
	double xn = 0;
	FS_TRY(sol_norm(s, x, &xn));
	memset(info, 0, sizeof(*info));
	info->rhs_norm = (float)h.rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)h.sol0;
	info->res_norm_initial = (float)h.res0;
	info->sol_norm_final = (float)xn;
	info->res_norm_final = (float)h.res;
	if (user_stop) {
		info->status = FS_CONVERGED_USER;
		info->iters = user_stop;
	}
	else {
		info->status = h.status;
		info->iters = h.info_iters;
		if (h.iter > 0 && info->iters == 0)
			info->status = FS_DIVERGED_ITERS;  // cg.hh:135-136
	}
	if (h.flags & KF_NONFINITE)
		return set_err(ctx, FS_ERR_NON_FINITE, "pipelined CG: non-finite residual norm");
	return FS_OK;
}

// ------------------------------------------- mixed precision refined CG --

// Classic iterative refinement: the residual, the update and the stopping
// test are FP64 (r = b - A x with the FP64 values), each correction
// A d = r is solved by FP32 Jacobi-PCG (FP32 values and vectors,
// compensated dots) to inner_rtol, and x += d in FP64.
static int cg_apply_mixed(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const int G = red_grid(ctx, n);
	const bool zg = s->set.base.use_zero_guess != 0;
	const int PK = s->dinv32() ? 1 : 0;
	double *r64 = s->w64[0];
	float *r32 = s->w32[0], *p32 = s->w32[1], *d32 = s->w32[3];
	const int maxiter = s->set.base.maxiter;
	FS_TRY(solver_hist(s, std::max(1, maxiter)));
	FS_TRY(init_state(s, s->st, (double)s->set.base.rtol, maxiter));
	FS_TRY(solver_norms(s, b, x, !zg, 0));
	if (zg) {
		k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
		FS_TRY(check_launch(ctx, "fill"));
	}
	auto residual = [&]() -> int {
		return launch_spmv<double, false, false>(
			ctx, s->A, s->A->val, (const double *)x->d, nullptr,
			EpiIrResidual{(const double *)b->d, r64, r32, s->st, s->part, s->counter});
	};
	FS_TRY(residual());
	FS_TRY(read_state(s));
	const double tol = s->hst->tol;
	const double res0 = s->hst->res;
	double res = res0;
	int total = 0, outer = 0;
	int status = FS_DIVERGED_ITERS;
	const double inner_rtol = s->set.inner_rtol > 0 ? s->set.inner_rtol : 1e-4;
	const int max_outer = s->set.max_outer > 0 ? s->set.max_outer : 64;
	const int k = k_default(s) > 1 ? k_default(s) : 32;
	std::vector<double> host_hist;
	while (true) {
		if (res < tol) {
			status = FS_CONVERGED_RTOL;
			break;
		}
		if (total >= maxiter || outer >= max_outer || !std::isfinite(res))
			break;
		// inner FP32 PCG on A d = r32, d0 = 0
		k_inner_init<<<1, 1, 0, ctx->stream>>>(s->st_in, s->st, inner_rtol, maxiter - total);
		FS_TRY(check_launch(ctx, "inner init"));
		k_fill<float><<<G, kThreads, 0, ctx->stream>>>(n, d32, 0.f);
		FS_TRY(check_launch(ctx, "fill"));
		if (PK)
			k_cg_start<float, 1><<<G, kThreads, 0, ctx->stream>>>(n, r32, s->dinv32(), p32, s->st_in, s->part, s->counter);
		else
			k_cg_start<float, 0><<<G, kThreads, 0, ctx->stream>>>(n, r32, nullptr, p32, s->st_in, s->part, s->counter);
		FS_TRY(check_launch(ctx, "inner start"));
		// the inner tolerance refers to ||r32||: k_cg_start sets res0 only
		CgArgs args{b, x, k};
		GraphKey key{b->d, x->d, 1000 + k * 2 + PK};
		int inner_iters = 0;
		for (int prev = -1;;) {
			FS_CUDA_TRY(ctx, cudaMemcpyAsync(s->hst, s->st_in, sizeof(KState), cudaMemcpyDeviceToHost, ctx->stream));
			FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
			if (s->hst->done || s->hst->iter == prev)
				break;
			prev = s->hst->iter;
			FS_TRY(graph_run(s, key, PK ? cg_body32<1> : cg_body32<0>, &args));
		}
		inner_iters = s->hst->iter;
		if (inner_iters == 0 && !s->hst->done)
			break;
		total += inner_iters;
		outer += 1;
		k_ir_update<<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, d32);
		FS_TRY(check_launch(ctx, "refinement update"));
		FS_TRY(residual());
		FS_TRY(read_state(s));
		res = s->hst->res;
		host_hist.push_back(res);
		if (s->diag && s->diag(s->diag_user, reinterpret_cast<fs_vec>(x), res)) {
			status = FS_CONVERGED_USER;
			break;
		}
		if (inner_iters == 0)
			break;
	}
	s->mixed_outer = outer;
	s->mixed_inner = total;
	// history: outer residuals (FP64) after each refinement step
	s->hhist.assign(host_hist.begin(), host_hist.end());
	s->hhist_count = -1;
	double xn = 0;
	FS_TRY(sol_norm(s, x, &xn));
	memset(info, 0, sizeof(*info));
	FS_TRY(read_state(s));
	info->rhs_norm = (float)s->hst->rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)s->hst->sol0;
	info->res_norm_initial = (float)res0;
	info->res_norm_final = (float)res;
	info->sol_norm_final = (float)xn;
	info->status = status;
	info->iters = status == FS_DIVERGED_ITERS ? 0 : total;
	info->restarts = outer;
	if (!std::isfinite(res))
		return set_err(ctx, FS_ERR_NON_FINITE, "mixed CG: non-finite residual norm");
	return FS_OK;
}

struct RcArgs {
	Vec *b, *x;
	int k;
	double delta;
};

template<int PK>
static int rc_body(Solver *s, void *a) {
	RcArgs *g = (RcArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	float *r = s->w32[0], *p = s->w32[1], *w = s->w32[2], *xs = s->w32[3];
	const float *dinv = s->dinv32();
	// four elements per thread and pass: a quarter of the grid
	const int G4 = grid_for(ctx, (n + 3) / 4, kThreads, 8);
	for (int k = 0; k < g->k; ++k) {
		FS_TRY(launch_spmv<float, false, false>(
			ctx, s->A, s->A->val32, p, nullptr,
			EpiCgAp<float>{w, p, s->st, s->part, s->counter}));
		FS_TRY(check_launch_rc(ctx,
		                       launch_pdl(ctx->stream, k_rc_resid4<PK>, G4, kThreads, 0, n, r, w, dinv,
		                                  s->st, s->part, s->counter, s->hist, g->delta),
		                       "reliable cg update"));
		FS_TRY(check_launch_rc(ctx, launch_pdl(ctx->stream, k_cg_dir_x<PK>, G4, kThreads, 0, n, p, r,
		                                       dinv, xs, (const KState *)s->st),
		                       "cg direction f32"));
	}
	return FS_OK;
}

// FP32 CG with FP64 reliable updates (residual replacement)
static int cg_apply_reliable(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const int G = red_grid(ctx, n);
	const bool zg = s->set.base.use_zero_guess != 0;
	const int PK = s->dinv32() ? 1 : 0;
	float *r32 = s->w32[0], *p32 = s->w32[1], *xs = s->w32[3];
	const float *dinv = s->dinv32();
	const int maxiter = s->set.base.maxiter;
	const double delta = s->set.inner_rtol > 0 ? s->set.inner_rtol : 0.1;
	const double rtol = (double)s->set.base.rtol;
	const bool head = s->set.fp64_head > rtol;
	FS_TRY(solver_hist(s, std::max(1, maxiter)));
	auto true_residual = [&]() -> int {
		return launch_spmv<double, false, false>(
			ctx, s->A, s->A->val, (const double *)x->d, nullptr,
			EpiRelResidual{(const double *)b->d, r32, s->st, s->part, s->counter});
	};
	int user_stop = 0;
	bool head_stop = false;  // the user stopped the FP64 head: x is final
	int64_t seen = 0;
	const int G4 = grid_for(ctx, (n + 3) / 4, kThreads, 8);
	if (head) {
		// FP64 PCG (the cg_apply64 iteration) to fp64_head * ||b||
		const size_t n64 = (size_t)((n + 31) / 32 * 32 + 32) * 8;
		for (int i = 0; i < 3; ++i)
			if (!s->w64[i])
				FS_TRY(dalloc(s, (void **)&s->w64[i], n64));
		double *r64 = s->w64[0], *p64 = s->w64[1];
		const int PK64 = s->dinv64() ? 1 : 0;
		FS_TRY(init_state(s, s->st, s->set.fp64_head, maxiter));
		FS_TRY(solver_norms(s, b, x, !zg, 0));
		if (zg) {
			k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
			FS_TRY(check_launch(ctx, "fill"));
			k_copy<double><<<G, kThreads, 0, ctx->stream>>>(n, (const double *)b->d, r64);
			FS_TRY(check_launch(ctx, "copy"));
		}
		else {
			FS_TRY(launch_spmv<double, false, false>(ctx, s->A, s->A->val, (const double *)x->d,
			                                         nullptr, EpiResidual<double>{(const double *)b->d, r64}));
		}
		if (PK64)
			k_cg_start<double, 1><<<G, kThreads, 0, ctx->stream>>>(n, r64, s->dinv64(), p64, s->st,
			                                                      s->part, s->counter);
		else
			k_cg_start<double, 0><<<G, kThreads, 0, ctx->stream>>>(n, r64, nullptr, p64, s->st,
			                                                      s->part, s->counter);
		FS_TRY(check_launch(ctx, "cg start"));
		FS_TRY(read_state(s));
		if (!s->hst->done) {
			CgArgs args{b, x, k_default(s)};
			LoopSpec L{x, {b->d, x->d, 0}, PK64 ? cg_body64<1> : cg_body64<0>, &args, nullptr,
			           &args.k, 4000 + PK64};
			FS_TRY(run_loop(s, L, &user_stop));
		}
		seen = s->hst->iter;
		head_stop = user_stop != 0;
		const bool go_on = !user_stop && s->hst->status == FS_CONVERGED_RTOL;
		if (go_on) {
			// continue the same process: the direction in FP32, the residual
			// replaced by the FP64 b - A x, beta from the last FP64 rho
			k_head_switch<<<1, 1, 0, ctx->stream>>>(s->st, rtol);
			FS_TRY(check_launch(ctx, "head switch"));
			k_to_f32<<<G, kThreads, 0, ctx->stream>>>(n, p64, p32);
			FS_TRY(check_launch(ctx, "direction to f32"));
			k_fill<float><<<G, kThreads, 0, ctx->stream>>>(n, xs, 0.f);
			FS_TRY(check_launch(ctx, "fill"));
			FS_TRY(true_residual());
			if (PK)
				k_rel_finish<1><<<G, kThreads, 0, ctx->stream>>>(n, r32, dinv, s->st, s->part, s->counter);
			else
				k_rel_finish<0><<<G, kThreads, 0, ctx->stream>>>(n, r32, nullptr, s->st, s->part,
				                                                s->counter);
			FS_TRY(check_launch(ctx, "head finish"));
			if (PK)
				k_cg_dir_x<1><<<G4, kThreads, 0, ctx->stream>>>(n, p32, r32, dinv, xs, s->st);
			else
				k_cg_dir_x<0><<<G4, kThreads, 0, ctx->stream>>>(n, p32, r32, nullptr, xs, s->st);
			FS_TRY(check_launch(ctx, "cg direction f32"));
		}
		// otherwise (user stop, maxiter, non-finite) the FP64 loop's verdict
		// stands and x holds its iterate
		FS_TRY(read_state(s));
	}
	else {
		FS_TRY(init_state(s, s->st, rtol, maxiter));
		FS_TRY(solver_norms(s, b, x, !zg, 0));
		if (zg) {
			k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
			FS_TRY(check_launch(ctx, "fill"));
		}
		k_fill<float><<<G, kThreads, 0, ctx->stream>>>(n, xs, 0.f);
		FS_TRY(check_launch(ctx, "fill"));
		FS_TRY(true_residual());
		if (PK)
			k_cg_start<float, 1><<<G, kThreads, 0, ctx->stream>>>(n, r32, dinv, p32, s->st, s->part,
			                                                     s->counter);
		else
			k_cg_start<float, 0><<<G, kThreads, 0, ctx->stream>>>(n, r32, nullptr, p32, s->st,
			                                                     s->part, s->counter);
		FS_TRY(check_launch(ctx, "cg start f32"));
		FS_TRY(read_state(s));
		// reference level for the first replacement = the initial residual
		KState h = *s->hst;
		h.aux[1] = h.res0;
		FS_CUDA_TRY(ctx, cudaMemcpyAsync(&s->st->aux[1], &h.aux[1], sizeof(double),
		                                 cudaMemcpyHostToDevice, ctx->stream));
		FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	}
	const double res0 = s->hst->res0;
	Chunk chunk(k_default(s) > 1 ? k_default(s) : 32);
	RcArgs args{b, x, chunk.k, delta};
	GraphKey key{b->d, x->d, 0};
	int64_t seg_start = s->hst->iter;  // iteration of the last replacement
	auto body = PK ? rc_body<1> : rc_body<0>;
	auto fold = [&]() -> int {
		// the last iteration's solution step is still pending
		k_rel_fold_pending<<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, xs, p32, s->st);
		return check_launch(ctx, "reliable fold");
	};
	while (!s->hst->done && !user_stop) {
		args.k = chunk.k;
		key.k = 2000 + 2 * chunk.k + PK;
		FS_TRY(graph_run(s, key, body, &args));
		FS_TRY(read_state(s));
		if (s->hst->flags & KF_RELIABLE) {
			chunk.restart(s->hst->iter - seg_start);
			seg_start = s->hst->iter;
		}
		else
			chunk.grow();
		if (s->hst->flags & KF_RELIABLE) {
			FS_TRY(fold());
			FS_TRY(true_residual());
			if (PK)
				k_rel_finish<1><<<G, kThreads, 0, ctx->stream>>>(n, r32, dinv, s->st, s->part, s->counter);
			else
				k_rel_finish<0><<<G, kThreads, 0, ctx->stream>>>(n, r32, nullptr, s->st, s->part,
				                                                s->counter);
			FS_TRY(check_launch(ctx, "reliable finish"));
			// the direction from the replaced residual; alpha_x is 0 here, so
			// xs (cleared by the fold) stays 0
			if (PK)
				k_cg_dir_x<1><<<G4, kThreads, 0, ctx->stream>>>(n, p32, r32, dinv, xs, s->st);
			else
				k_cg_dir_x<0><<<G4, kThreads, 0, ctx->stream>>>(n, p32, r32, nullptr, xs, s->st);
			FS_TRY(check_launch(ctx, "cg direction f32"));
			FS_TRY(read_state(s));
		}
		if (s->diag) {
			int64_t nh = std::min<int64_t>(s->hst->iter, s->hist_cap);
			std::vector<double> hh(nh > seen ? nh - seen : 0);
			if (!hh.empty())
				FS_CUDA_TRY(ctx, cudaMemcpy(hh.data(), s->hist + seen, hh.size() * sizeof(double),
				                            cudaMemcpyDeviceToHost));
			for (size_t j = 0; j < hh.size() && !user_stop; ++j)
				if (s->diag(s->diag_user, reinterpret_cast<fs_vec>(x), hh[j]))
					user_stop = (int)(seen + j + 1);
			seen = nh;
			if (user_stop)
				break;
		}
	}
	if (user_stop && !head_stop)
		FS_TRY(fold());
	KState &h = *s->hst;
	s->hhist_count = std::min<int64_t>(h.iter, s->hist_cap);
	s->mixed_outer = h.restarts;
	s->mixed_inner = h.iter;
	double xn = 0;
	FS_TRY(sol_norm(s, x, &xn));
	memset(info, 0, sizeof(*info));
	info->rhs_norm = (float)h.rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)h.sol0;
	info->res_norm_initial = (float)res0;
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
	}
	if (h.flags & KF_NONFINITE)
		return set_err(ctx, FS_ERR_NON_FINITE, "mixed CG: non-finite residual norm");
	return FS_OK;
}

// ------------------------------------------------------ BiCGSTAB apply --

struct BiArgs {
	Vec *b, *x;
	int k;
};

template<int PK>
static int bi_body64(Solver *s, void *a) {
	BiArgs *g = (BiArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	double *res = s->w64[0], *rt = s->w64[1], *p = s->w64[2], *v = s->w64[3],
	       *sv = s->w64[4], *t = s->w64[5];
	double *x = (double *)g->x->d;
	const double *dinv = s->dinv64();
	const int G = red_grid(ctx, n);
	for (int k = 0; k < g->k; ++k) {
		k_bi_p<double><<<G, kThreads, 0, ctx->stream>>>(n, p, v, res, s->st);
		FS_TRY(check_launch(ctx, "bicgstab p"));
		if (PK)
			FS_TRY((launch_spmv<double, false, true>(ctx, s->A, s->A->val, p, dinv,
			                                         EpiBiV<double>{v, rt, s->st, s->part, s->counter})));
		else
			FS_TRY((launch_spmv<double, false, false>(ctx, s->A, s->A->val, p, nullptr,
			                                          EpiBiV<double>{v, rt, s->st, s->part, s->counter})));
		k_bi_s<double><<<G, kThreads, 0, ctx->stream>>>(n, sv, v, res, s->st, s->part, s->counter);
		FS_TRY(check_launch(ctx, "bicgstab s"));
		if (PK)
			FS_TRY((launch_spmv<double, false, true>(ctx, s->A, s->A->val, sv, dinv,
			                                         EpiBiT<double>{t, sv, s->st, s->part, s->counter})));
		else
			FS_TRY((launch_spmv<double, false, false>(ctx, s->A, s->A->val, sv, nullptr,
			                                          EpiBiT<double>{t, sv, s->st, s->part, s->counter})));
		k_bi_x<double, PK><<<G, kThreads, 0, ctx->stream>>>(n, x, p, sv, t, res, rt, dinv, s->st,
		                                                   s->part, s->counter, s->hist);
		FS_TRY(check_launch(ctx, "bicgstab x"));
	}
	return FS_OK;
}

static int bi_restart(Solver *s, void *a) {
	BiArgs *g = (BiArgs *)a;
	Ctx *ctx = s->ctx;
	double *res = s->w64[0], *rt = s->w64[1], *p = s->w64[2];
	FS_TRY(launch_spmv<double, false, false>(ctx, s->A, s->A->val, (const double *)g->x->d, nullptr,
	                                         EpiResidual<double>{(const double *)g->b->d, res}));
	k_bi_restart<double><<<red_grid(ctx, s->n), kThreads, 0, ctx->stream>>>(s->n, res, rt, p, s->st,
	                                                                       s->part, s->counter);
	return check_launch(ctx, "bicgstab restart");
}

static int bicgstab_apply64(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const int G = red_grid(ctx, n);
	const bool zg = s->set.base.use_zero_guess != 0;
	const int PK = s->dinv64() ? 1 : 0;
	double *res = s->w64[0], *rt = s->w64[1], *p = s->w64[2], *v = s->w64[3];
	FS_TRY(solver_hist(s, std::max(1, s->set.base.maxiter)));
	FS_TRY(init_state(s, s->st, (double)s->set.base.rtol, s->set.base.maxiter));
	FS_TRY(solver_norms(s, b, x, !zg, 0));
	if (zg) {
		k_copy<double><<<G, kThreads, 0, ctx->stream>>>(n, (const double *)b->d, res);
		FS_TRY(check_launch(ctx, "copy"));
		k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
		FS_TRY(check_launch(ctx, "fill"));
	}
	else {
		FS_TRY(launch_spmv<double, false, false>(ctx, s->A, s->A->val, (const double *)x->d, nullptr,
		                                         EpiResidual<double>{(const double *)b->d, res}));
	}
	k_bi_start<double><<<G, kThreads, 0, ctx->stream>>>(n, res, rt, p, v, s->st, s->part, s->counter);
	FS_TRY(check_launch(ctx, "bicgstab start"));
	FS_TRY(read_state(s));
	int user_stop = 0;
	if (!s->hst->done) {
		BiArgs args{b, x, k_default(s)};
		LoopSpec L{x, {b->d, x->d, 0}, PK ? bi_body64<1> : bi_body64<0>, &args, bi_restart, &args.k,
		           100 + PK};
		FS_TRY(run_loop(s, L, &user_stop));
	}
	KState &h = *s->hst;
	s->hhist_count = std::min<int64_t>((int64_t)h.nhist, s->hist_cap);
	double xn = 0;
	FS_TRY(sol_norm(s, x, &xn));
	memset(info, 0, sizeof(*info));
	info->rhs_norm = (float)h.rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)h.sol0;
	info->res_norm_initial = (float)h.res0;
	info->sol_norm_final = (float)xn;
	info->res_norm_final = (float)h.res;
	info->restarts = h.restarts;
	if (user_stop) {
		info->status = FS_CONVERGED_USER;
		info->iters = user_stop;
	}
	else {
		info->status = h.status;
		info->iters = h.info_iters;
		if (h.res0 >= h.tol && info->iters == 0)
			info->status = FS_DIVERGED_ITERS;  // bicgstab.hh:183-184
	}
	if (h.flags & KF_ALPHA_ZERO)
		return set_err(ctx, FS_ERR_BREAKDOWN, "BiCGSTAB: encountered alpha = 0 (bicgstab.hh:129)");
	if (h.flags & KF_NONFINITE)
		return set_err(ctx, FS_ERR_NON_FINITE, "BiCGSTAB: non-finite residual norm");
	return FS_OK;
}

// ------------------------------------------- mixed precision BiCGSTAB --

template<int PK>
static int bi_body32(Solver *s, void *a) {
	BiArgs *g = (BiArgs *)a;
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	float *res = s->w32[0], *rt = s->w32[1], *p = s->w32[2], *v = s->w32[3], *sv = s->w32[4],
	      *t = s->w32[5], *xs = s->w32[6];
	const float *dinv = s->dinv32();
	const int G = red_grid(ctx, n);
	for (int k = 0; k < g->k; ++k) {
		k_bi_p<float><<<G, kThreads, 0, ctx->stream>>>(n, p, v, res, s->st);
		FS_TRY(check_launch(ctx, "bicgstab p f32"));
		if (PK)
			FS_TRY((launch_spmv<float, false, true>(ctx, s->A, s->A->val32, p, dinv,
			                                        EpiBiV<float>{v, rt, s->st, s->part, s->counter})));
		else
			FS_TRY((launch_spmv<float, false, false>(ctx, s->A, s->A->val32, p, nullptr,
			                                         EpiBiV<float>{v, rt, s->st, s->part, s->counter})));
		k_bi_s<float><<<G, kThreads, 0, ctx->stream>>>(n, sv, v, res, s->st, s->part, s->counter);
		FS_TRY(check_launch(ctx, "bicgstab s f32"));
		if (PK)
			FS_TRY((launch_spmv<float, false, true>(ctx, s->A, s->A->val32, sv, dinv,
			                                        EpiBiT<float>{t, sv, s->st, s->part, s->counter})));
		else
			FS_TRY((launch_spmv<float, false, false>(ctx, s->A, s->A->val32, sv, nullptr,
			                                         EpiBiT<float>{t, sv, s->st, s->part, s->counter})));
		k_bi_x<float, PK, true><<<G, kThreads, 0, ctx->stream>>>(n, xs, p, sv, t, res, rt, dinv, s->st,
		                                                        s->part, s->counter, s->hist);
		FS_TRY(check_launch(ctx, "bicgstab x f32"));
	}
	return FS_OK;
}

// FP32 BiCGSTAB recurrences on a correction xs, with the FP64 residual
// b - A x replacing the recurrence residual whenever it has dropped by
// inner_rtol since the last replacement and at every stop, so that the
// stopping test is the reference's, on the FP64 residual.
static int bicgstab_apply_reliable(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Ctx *ctx = s->ctx;
	const int64_t n = s->n;
	const int G = red_grid(ctx, n);
	const bool zg = s->set.base.use_zero_guess != 0;
	const int PK = s->dinv32() ? 1 : 0;
	float *res = s->w32[0], *rt = s->w32[1], *p = s->w32[2], *v = s->w32[3], *xs = s->w32[6];
	const int maxiter = s->set.base.maxiter;
	const double delta = s->set.inner_rtol > 0 ? s->set.inner_rtol : 1e-2;
	FS_TRY(solver_hist(s, std::max(1, maxiter)));
	FS_TRY(init_state(s, s->st, (double)s->set.base.rtol, maxiter));
	FS_TRY(solver_norms(s, b, x, !zg, 0));
	if (zg) {
		k_fill<double><<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, 0.0);
		FS_TRY(check_launch(ctx, "fill"));
	}
	auto fold_and_residual = [&]() -> int {
		k_rel_fold<<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, xs);
		FS_TRY(check_launch(ctx, "fold"));
		return launch_spmv<double, false, false>(
			ctx, s->A, s->A->val, (const double *)x->d, nullptr,
			EpiRelResidual{(const double *)b->d, res, s->st, s->part, s->counter});
	};
	k_fill<float><<<G, kThreads, 0, ctx->stream>>>(n, xs, 0.f);
	FS_TRY(check_launch(ctx, "fill"));
	FS_TRY(fold_and_residual());
	k_bi_start<float><<<G, kThreads, 0, ctx->stream>>>(n, res, rt, p, v, s->st, s->part, s->counter);
	FS_TRY(check_launch(ctx, "bicgstab start f32"));
	FS_TRY(read_state(s));
	const double res0 = s->hst->res0;
	{
		double a[2] = {delta, res0};  // aux[0] = replacement factor, aux[1] = level
		FS_CUDA_TRY(ctx, cudaMemcpyAsync(&s->st->aux[0], a, sizeof a, cudaMemcpyHostToDevice, ctx->stream));
		FS_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
	}
	int user_stop = 0;
	int64_t seen = 0;
	const int k = k_default(s) > 1 ? k_default(s) : 32;
	BiArgs args{b, x, k};
	GraphKey key{b->d, x->d, 400 + k * 2 + PK};
	while (!s->hst->done && !user_stop) {
		FS_TRY(graph_run(s, key, PK ? bi_body32<1> : bi_body32<0>, &args));
		FS_TRY(read_state(s));
		if (s->hst->flags & KF_RELIABLE) {
			FS_TRY(fold_and_residual());
			k_bi_rel_decide<<<1, 1, 0, ctx->stream>>>(s->st);
			FS_TRY(check_launch(ctx, "bicgstab decide"));
			k_bi_rho<float><<<G, kThreads, 0, ctx->stream>>>(n, rt, res, s->st, s->part, s->counter);
			FS_TRY(check_launch(ctx, "bicgstab rho"));
			FS_TRY(read_state(s));
		}
		if ((s->hst->flags & KF_RESTART) && !s->hst->done) {
			// bicgstab.hh:103-113 (also after a spent recurrence): r from the
			// FP64 residual, r~ = r, p = r
			FS_TRY(fold_and_residual());
			k_bi_restart<float><<<G, kThreads, 0, ctx->stream>>>(n, res, rt, p, s->st, s->part, s->counter);
			FS_TRY(check_launch(ctx, "bicgstab restart f32"));
			FS_TRY(read_state(s));
		}
		if (s->diag) {
			const int64_t nh = std::min<int64_t>(s->hst->nhist, s->hist_cap);
			std::vector<double> hh(nh > seen ? nh - seen : 0);
			if (!hh.empty())
				FS_CUDA_TRY(ctx, cudaMemcpy(hh.data(), s->hist + seen, hh.size() * sizeof(double),
				                            cudaMemcpyDeviceToHost));
			for (size_t j = 0; j < hh.size() && !user_stop; ++j)
				if (s->diag(s->diag_user, reinterpret_cast<fs_vec>(x), hh[j]))
					user_stop = (int)(seen + j + 1);
			seen = nh;
		}
	}
	k_rel_fold<<<G, kThreads, 0, ctx->stream>>>(n, (double *)x->d, xs);
	FS_TRY(check_launch(ctx, "fold"));
	FS_TRY(read_state(s));
	KState &h = *s->hst;
	s->hhist_count = std::min<int64_t>(h.nhist, s->hist_cap);
	s->mixed_outer = h.restarts;
	s->mixed_inner = h.iter;
	double xn = 0;
	FS_TRY(sol_norm(s, x, &xn));
	memset(info, 0, sizeof(*info));
	info->rhs_norm = (float)h.rhs_norm;
	info->sol_norm_initial = zg ? 0.f : (float)h.sol0;
	info->res_norm_initial = (float)res0;
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
		if (res0 >= h.tol && info->iters == 0)
			info->status = FS_DIVERGED_ITERS;
	}
	if (h.flags & KF_NONFINITE)
		return set_err(ctx, FS_ERR_NON_FINITE, "mixed BiCGSTAB: non-finite residual norm");
	return FS_OK;
}

int ensure_transpose(Csr *A);
int gmres_apply(Solver *s, Vec *b, Vec *x, fs_solve_info *info);
int gmres_apply_mixed(Solver *s, Vec *b, Vec *x, fs_solve_info *info);

}  // namespace fsg

using namespace fsg;

// ================================================================ C ABI ==

extern "C" {

FS_API int fs_krylov_settings_default(fs_krylov_settings *s) {
	if (!s)
		return FS_ERR_INVALID_ARG;
	memset(s, 0, sizeof(*s));
	s->base.maxiter = 1000;
	s->base.rtol = 0.f;
	s->base.atol = 0.f;
	s->base.use_zero_guess = 1;
	s->max_krylov_dim = -1;
	s->pre_side = FS_RIGHT;
	s->restart = 0;
	s->ortho = FS_ORTHO_AUTO;
	s->k_readback = 0;
	s->refine = FS_REFINE_RELIABLE;
	s->inner_rtol = 0.0;  // per-method default
	s->max_outer = 64;
	s->fp64_head = 3e-3;
	return FS_OK;
}

FS_API int fs_krylov_create(fs_ctx h, int method, const fs_krylov_settings *set, fs_csr Ah,
                            const fs_precond *P, fs_solver *out) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Csr *A = reinterpret_cast<Csr *>(Ah);
	if (!ok_ctx(ctx) || !ok_csr(A) || !out || !set)
		return FS_ERR_BAD_HANDLE;
	*out = nullptr;
	if (method < FS_CG || method > FS_CG_PIPELINED)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_krylov_create: unknown method %d", method);
	if (A->nrows != A->ncols)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_krylov_create: operator must be square");
	Solver *s = new Solver();
	s->ctx = ctx;
	s->method = method;
	s->set = *set;
	s->A = A;
	s->n = A->nrows;
	if (P) {
		s->P.kind = P->kind;
		if (P->kind == FS_PRECOND_DIAG) {
			Vec *d = reinterpret_cast<Vec *>(P->diag);
			if (!ok_vec(d) || d->n != A->nrows) {
				delete s;
				return set_err(ctx, FS_ERR_BAD_HANDLE, "fs_krylov_create: bad diagonal preconditioner");
			}
			s->P.diag = d;
		}
		else if (P->kind == FS_PRECOND_CSR) {
			// a CSR preconditioner whose entries are all on the diagonal (the
			// D^-1 operator of util/test/mesh.hh:123-140) becomes a diagonal
			// vector fused into the device loops; any other operator is
			// applied as its own step (generic.cu)
			Csr *M = reinterpret_cast<Csr *>(P->op);
			if (!ok_csr(M) || M->nrows != A->nrows || M->ncols != A->nrows || M->ctx != ctx) {
				delete s;
				return set_err(ctx, FS_ERR_BAD_HANDLE, "fs_krylov_create: bad CSR preconditioner");
			}
			bool diagonal = !stores_no_rows(M);
			if (diagonal) {
				std::vector<int> hc(M->nnz);
				if (M->nnz)
					cudaMemcpy(hc.data(), M->col, M->nnz * sizeof(int), cudaMemcpyDeviceToHost);
				for (int64_t i = 0; i < M->nrows && diagonal; ++i)
					for (int k = M->h_rowptr[i]; k < M->h_rowptr[i + 1]; ++k)
						if (hc[k] != i)
							diagonal = false;
			}
			s->P.kind = FS_PRECOND_CSR;
			s->P.op = M;
			s->pc_diagonal = diagonal;
		}
		else if (P->kind == FS_PRECOND_SOLVER) {
			Solver *inner = reinterpret_cast<Solver *>(P->solver);
			if (!ok_slv(inner) || inner->n != A->nrows || inner->ctx != ctx || inner == s) {
				delete s;
				return set_err(ctx, FS_ERR_BAD_HANDLE, "fs_krylov_create: bad solver preconditioner");
			}
			s->P.solver = inner;
		}
		else if (P->kind != FS_PRECOND_NONE && P->kind != FS_PRECOND_JACOBI) {
			delete s;
			return set_err(ctx, FS_ERR_INVALID_ARG, "fs_krylov_create: unknown preconditioner kind");
		}
	}
	if (s->P.kind == FS_PRECOND_JACOBI && A->shell_fn) {
		delete s;
		return set_err(ctx, FS_ERR_INVALID_ARG,
		               "fs_krylov_create: Jacobi needs the operator's diagonal; a shell operator stores none");
	}
	const bool mixed_method =
		method == FS_CG_MIXED || method == FS_BICGSTAB_MIXED || method == FS_GMRES_MIXED;
	if (mixed_method && (A->shell_fn || (s->P.kind == FS_PRECOND_CSR && !s->pc_diagonal) ||
	                     s->P.kind == FS_PRECOND_SOLVER)) {
		delete s;
		return set_err(ctx, FS_ERR_UNSUPPORTED,
		               "fs_krylov_create: mixed-precision solvers take a stored or matrix-free "
		               "operator and an identity, Jacobi or diagonal preconditioner");
	}
	if (method == FS_GMRES || method == FS_GMRES_MIXED) {
		int m = set->max_krylov_dim < 0 ? set->base.maxiter : set->max_krylov_dim;
		if (m > 100 || (!set->restart && set->base.maxiter > m)) {
			delete s;
			return set_err(ctx, FS_ERR_BREAKDOWN,
			               "GMRES settings fail the reference's validate() (gmres.hh:394-404)");
		}
	}
	int st = solver_alloc(s);
	if (st == FS_OK && (s->P.kind == FS_PRECOND_DIAG ||
	                    (s->P.kind == FS_PRECOND_CSR && s->pc_diagonal))) {
		// copy the diagonal into the solver (FP64 + FP32)
		if (s->P.kind == FS_PRECOND_CSR) {
			Csr *M = s->P.op;
			// diagonal entries in row order: the values array itself, with
			// zeros where a row has no entry
			std::vector<double> hv(M->nnz), dv(s->n, 0.0);
			if (M->nnz)
				cudaMemcpy(hv.data(), M->val, M->nnz * sizeof(double), cudaMemcpyDeviceToHost);
			for (int64_t i = 0; i < s->n; ++i)
				for (int k = M->h_rowptr[i]; k < M->h_rowptr[i + 1]; ++k)
					dv[i] = hv[k];
			if (s->n)
				cudaMemcpy(s->w64[10], dv.data(), s->n * sizeof(double), cudaMemcpyHostToDevice);
			s->P.kind = FS_PRECOND_DIAG;
		}
		else {
			Vec *d = s->P.diag;
			if (d->dtype == FS_F64)
				cudaMemcpyAsync(s->w64[10], d->d, s->n * 8, cudaMemcpyDeviceToDevice, ctx->stream);
			else {
				std::vector<float> hf(s->n);
				std::vector<double> hd(s->n);
				cudaMemcpy(hf.data(), d->d, s->n * 4, cudaMemcpyDeviceToHost);
				for (int64_t i = 0; i < s->n; ++i)
					hd[i] = hf[i];
				cudaMemcpy(s->w64[10], hd.data(), s->n * 8, cudaMemcpyHostToDevice);
			}
		}
		std::vector<double> hd(s->n);
		std::vector<float> hf(s->n);
		cudaStreamSynchronize(ctx->stream);
		if (s->n)
			cudaMemcpy(hd.data(), s->w64[10], s->n * 8, cudaMemcpyDeviceToHost);
		for (int64_t i = 0; i < s->n; ++i)
			hf[i] = (float)hd[i];
		if (s->n)
			cudaMemcpy(s->w32[10], hf.data(), s->n * 4, cudaMemcpyHostToDevice);
		fence_setup_copies();
		if (cudaGetLastError() != cudaSuccess)
			st = set_err(ctx, FS_ERR_CUDA, "fs_krylov_create: preconditioner copy failed");
	}
	if (st != FS_OK) {
		for (void *p : s->bufs)
			cudaFree(p);
		if (s->hst)
			cudaFreeHost(s->hst);
		delete s;
		return st;
	}
	*out = reinterpret_cast<fs_solver>(s);
	return FS_OK;
}

FS_API int fs_krylov_destroy(fs_solver h) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s))
		return FS_ERR_BAD_HANDLE;
	cudaStreamSynchronize(s->ctx->stream);
	clear_graphs(s);
	for (void *p : s->bufs)
		cudaFree(p);
	if (s->AT) {
		if (s->AT->val32)
			cudaFree(s->AT->val32);  // the only array the view owns
		s->AT->magic = 0;
		delete s->AT;
	}
	if (s->basis)
		cudaFree(s->basis);
	if (s->hist)
		cudaFree(s->hist);
	if (s->hst)
		cudaFreeHost(s->hst);
	s->magic = 0;
	delete s;
	return FS_OK;
}

FS_API int fs_krylov_set_diagnostic(fs_solver h, fs_diag_fn fn, void *user) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s))
		return FS_ERR_BAD_HANDLE;
	s->diag = fn;
	s->diag_user = user;
	return FS_OK;
}

FS_API int fs_krylov_settings_get(fs_solver h, fs_krylov_settings *out) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s) || !out)
		return FS_ERR_BAD_HANDLE;
	*out = s->set;
	return FS_OK;
}

FS_API int fs_krylov_settings_set(fs_solver h, const fs_krylov_settings *in) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s) || !in)
		return FS_ERR_BAD_HANDLE;
	if (s->method == FS_GMRES || s->method == FS_GMRES_MIXED) {
		int m = in->max_krylov_dim < 0 ? in->base.maxiter : in->max_krylov_dim;
		if (m > 100 || (!in->restart && in->base.maxiter > m))
			return set_err(s->ctx, FS_ERR_BREAKDOWN,
			               "GMRES settings fail the reference's validate() (gmres.hh:394-404)");
	}
	cudaStreamSynchronize(s->ctx->stream);
	clear_graphs(s);
	s->set = *in;
	return FS_OK;
}

FS_API int fs_krylov_apply(fs_solver h, fs_vec bh, fs_vec xh, fs_solve_info *info) {
	Solver *s = reinterpret_cast<Solver *>(h);
	Vec *b = reinterpret_cast<Vec *>(bh), *x = reinterpret_cast<Vec *>(xh);
	if (!ok_slv(s) || !ok_vec(b) || !ok_vec(x) || !info)
		return FS_ERR_BAD_HANDLE;
	Ctx *ctx = s->ctx;
	if (b->n != s->n || x->n != s->n)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_krylov_apply: vector size %lld/%lld != %lld",
		               (long long)b->n, (long long)x->n, (long long)s->n);
	if (b->dtype != FS_F64 || x->dtype != FS_F64)
		return set_err(ctx, FS_ERR_UNSUPPORTED, "fs_krylov_apply: b and x must be FP64");
	if (b == x)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_krylov_apply: b and x must differ");
	cudaSetDevice(ctx->device);
	s->mixed_outer = s->mixed_inner = 0;
	if (needs_generic(s))
		return generic_apply(s, b, x, info);
	// the operator's values may have changed since the last apply
	// (fs_csr_update_values, fs_fv_assemble): derived arrays are rebuilt in
	// place, so captured graphs stay valid
	if (s->P.kind == FS_PRECOND_JACOBI)
		FS_TRY(ensure_dinv(s->A));
	const bool mixed =
		s->method == FS_CG_MIXED || s->method == FS_BICGSTAB_MIXED || s->method == FS_GMRES_MIXED;
	if (mixed)
		FS_TRY(ensure_val32(s->A));
	FS_TRY(ensure_sym(s->A, false));
	if (mixed)
		FS_TRY(ensure_sym(s->A, true));
	switch (s->method) {
	case FS_CG: return cg_apply64(s, b, x, info);
	case FS_CG_PIPELINED: return cg_apply_pipelined(s, b, x, info);
	case FS_BICGSTAB: return bicgstab_apply64(s, b, x, info);
	case FS_GMRES: return gmres_apply(s, b, x, info);
	case FS_CG_MIXED:
		return s->set.refine == FS_REFINE_RELIABLE ? cg_apply_reliable(s, b, x, info)
		                                          : cg_apply_mixed(s, b, x, info);
	case FS_BICGSTAB_MIXED: return bicgstab_apply_reliable(s, b, x, info);
	case FS_GMRES_MIXED: return gmres_apply_mixed(s, b, x, info);
	}
	return FS_ERR_INVALID_ARG;
}

// A^T x = b with the bound solver's method, settings and preconditioner
// (the Jacobi diagonal of A^T is A's).  The transposed operator is a view of
// A's CSC arrays, refreshed from A's current values on every call.
FS_API int fs_krylov_apply_transpose(fs_solver h, fs_vec bh, fs_vec xh, fs_solve_info *info) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s))
		return FS_ERR_BAD_HANDLE;
	Csr *A = s->A;
	FS_TRY(ensure_transpose(A));
	FS_TRY(ensure_dinv(A));
	if (!s->AT) {
		s->AT = new Csr();
		s->AT->ctx = A->ctx;
		s->AT->view = true;
	}
	Csr *T = s->AT;
	T->nrows = A->ncols;
	T->ncols = A->nrows;
	T->nnz = A->nnz;
	T->rowptr = A->t_colptr;
	T->col = A->t_row;
	T->val = A->t_val;
	T->blk = A->t_blk;
	T->blkinfo = A->t_blkinfo;
	T->nblk = A->t_nblk;
	T->dinv = A->dinv;
	T->dinv32 = A->dinv32;
	T->dinv_valid = true;
	T->val32_valid = false;  // rebuilt from the current values when needed
	if (s->method == FS_CG_MIXED || s->method == FS_BICGSTAB_MIXED || s->method == FS_GMRES_MIXED)
		FS_TRY(ensure_val32(T));
	s->A = T;
	int st = fs_krylov_apply(h, bh, xh, info);
	s->A = A;
	return st;
}

FS_API int fs_krylov_history(fs_solver h, double *hist, int64_t *n) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s) || !n)
		return FS_ERR_BAD_HANDLE;
	if (s->hhist_count < 0) {
		int64_t m = std::min<int64_t>(*n, (int64_t)s->hhist.size());
		if (hist && m > 0)
			memcpy(hist, s->hhist.data(), m * sizeof(double));
		*n = m;
		return FS_OK;
	}
	int64_t m = std::min<int64_t>(*n, s->hhist_count);
	if (hist && m > 0)
		FS_CUDA_TRY(s->ctx, cudaMemcpy(hist, s->hist, m * sizeof(double), cudaMemcpyDeviceToHost));
	*n = m;
	return FS_OK;
}

FS_API int fs_krylov_mixed_stats(fs_solver h, int *outer, int *inner) {
	Solver *s = reinterpret_cast<Solver *>(h);
	if (!ok_slv(s))
		return FS_ERR_BAD_HANDLE;
	if (outer) *outer = s->mixed_outer;
	if (inner) *inner = s->mixed_inner;
	return FS_OK;
}

}  // extern "C"
