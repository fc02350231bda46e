// Host-stepped Krylov loops for any operator and any preconditioner.
//
// The fused device loops (krylov.cu, gmres.cu) take a stored or matrix-free
// operator and an identity, Jacobi or diagonal preconditioner.  flecsolve's
// solvers take any op::base operator as A and any operator as P
// (solvers/krylov_parameters.hh:41-78): a caller's shell
// (operators/shell.hh:26-95), a general matrix, a nested solver.  For those,
// the loops below restate the reference's loops operation for operation --
// CG (solvers/cg.hh:43-139), the flexible CG (cg.hh:145-244), BiCGSTAB
// (bicgstab.hh:39-187) and restarted GMRES (gmres.hh:54-348) -- over device
// vectors.  Every vector operation is one call of the device vector
// policy, every reduction is the context's deterministic device reduction
// read back by the host (the reference's `.get()`), and every operator
// application is the operator's own: an SpMV with the reference's row
// arithmetic, the caller's callback, or the nested solver's apply.  The
// GMRES least-squares problem stays on the host, as in the reference.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "solver.cuh"

namespace fsg {
namespace {

fs_vec hv(Vec *v) { return reinterpret_cast<fs_vec>(v); }

struct Gen {
	Solver *s;
	Ctx *ctx;
	int64_t n;
	Vec dv;            // the Jacobi or diagonal preconditioner as a vector
	std::vector<double> hist;

	explicit Gen(Solver *s_) : s(s_), ctx(s_->ctx), n(s_->n) {}

	// work vector i of the solver (allocated on first use, kept)
	int vec(int i, Vec **out) {
		while ((int)s->gwork.size() <= i) {
			void *d = nullptr;
			const size_t bytes = (size_t)((n + 31) / 32 * 32 + 32) * 8;
			FS_CUDA_TRY(ctx, cudaMalloc(&d, bytes));
			s->bufs.push_back(d);
			FS_CUDA_TRY(ctx, cudaMemsetAsync(d, 0, bytes, ctx->stream));
			auto v = std::make_unique<Vec>();
			v->ctx = ctx;
			v->n = n;
			v->dtype = FS_F64;
			v->d = d;
			v->owns = false;
			s->gwork.push_back(std::move(v));
		}
		*out = s->gwork[i].get();
		return FS_OK;
	}

	int setup() {
		dv.ctx = ctx;
		dv.n = n;
		dv.dtype = FS_F64;
		dv.owns = false;
		dv.d = nullptr;
		if (s->P.kind == FS_PRECOND_JACOBI) {
			FS_TRY(ensure_dinv(s->A));
			dv.d = s->A->dinv;
		}
		else if (s->P.kind == FS_PRECOND_DIAG)
			dv.d = s->w64[10];
		return FS_OK;
	}

	// y = A x: the reference's row arithmetic for a stored matrix (the
	// products rounded and summed left to right, matrices/seq.hh:177-193)
	int apply_op(Csr *M, Vec *x, Vec *y) {
		if (M->shell_fn)
			return shell_apply(M, x, y);
		return fs_csr_spmv(reinterpret_cast<fs_csr>(M), hv(x), hv(y),
		                   M->fvm ? FS_SPMV_FMA : FS_SPMV_EXACT);
	}
	int A(Vec *x, Vec *y) { return apply_op(s->A, x, y); }

	// z = P r
	int P(Vec *r, Vec *z) {
		switch (s->P.kind) {
		case FS_PRECOND_NONE: return fs_vec_copy(hv(r), hv(z));
		case FS_PRECOND_JACOBI:
		case FS_PRECOND_DIAG: return fs_vec_multiply(hv(&dv), hv(r), hv(z));
		case FS_PRECOND_CSR: return apply_op(s->P.op, r, z);
		case FS_PRECOND_SOLVER: {
			fs_solve_info inner;
			return fs_krylov_apply(reinterpret_cast<fs_solver>(s->P.solver), hv(r), hv(z), &inner);
		}
		}
		return set_err(ctx, FS_ERR_INVALID_ARG, "unknown preconditioner kind");
	}

	// r = b - A x (operators/core.hh:129-142)
	int residual(Vec *b, Vec *x, Vec *r) {
		FS_TRY(A(x, r));
		return fs_vec_subtract(hv(b), hv(r), hv(r));
	}
	int dot(Vec *x, Vec *y, double *out) { return fs_vec_dot(hv(x), hv(y), out); }
	int norm(Vec *x, double *out) { return fs_vec_l2norm(hv(x), out); }
	int axpy(double a, Vec *x, Vec *y, Vec *z) { return fs_vec_axpy(a, hv(x), hv(y), hv(z)); }
	int copy(Vec *src, Vec *dst) { return fs_vec_copy(hv(src), hv(dst)); }

	// the residual norm handed to the diagnostic; nonzero *stop: the user
	// stops the solve
	int diag(Vec *x, double res, int *stop) {
		hist.push_back(res);
		*stop = 0;
		if (s->diag)
			*stop = s->diag(s->diag_user, hv(x), res) != 0;
		return FS_OK;
	}

	int check_finite(double v) {
		return std::isfinite(v) ? FS_OK
		                        : set_err(ctx, FS_ERR_NON_FINITE, "non-finite residual norm");
	}

	void finish() {
		s->hhist.assign(hist.begin(), hist.end());
		s->hhist_count = -1;
	}
};

// ------------------------------------------------------------- CG --
// cg.hh:43-139
int gen_cg(Gen &g, Vec *b, Vec *x, fs_solve_info *info) {
	const auto &set = g.s->set.base;
	Vec *r, *z, *p, *w;
	FS_TRY(g.vec(0, &r));
	FS_TRY(g.vec(1, &z));
	FS_TRY(g.vec(2, &p));
	FS_TRY(g.vec(3, &w));
	double b_norm;
	FS_TRY(g.norm(b, &b_norm));
	if (b_norm == 0.0)
		b_norm = 1.0;
	const double tol = set.rtol * b_norm;
	info->rhs_norm = (float)b_norm;
	if (set.use_zero_guess) {
		info->sol_norm_initial = 0;
		FS_TRY(fs_vec_set_scalar(hv(x), 0.0));
		FS_TRY(g.copy(b, r));
	}
	else {
		double xn;
		FS_TRY(g.norm(x, &xn));
		info->sol_norm_initial = (float)xn;
		FS_TRY(g.residual(b, x, r));
	}
	double res;
	FS_TRY(g.norm(r, &res));
	info->res_norm_initial = (float)res;
	if (res < tol) {
		info->res_norm_final = (float)res;
		info->status = FS_CONVERGED_RTOL;
		return FS_OK;
	}
	FS_TRY(g.P(r, z));
	double rho1, rho0;
	FS_TRY(g.dot(z, r, &rho1));
	rho0 = rho1;
	FS_TRY(g.copy(z, p));
	for (int iter = 0; iter < set.maxiter; ++iter) {
		FS_TRY(g.A(p, w));
		double alpha;
		FS_TRY(g.dot(w, p, &alpha));
		alpha = rho1 / alpha;
		FS_TRY(g.axpy(alpha, p, x, x));
		FS_TRY(g.axpy(-alpha, w, r, r));
		FS_TRY(g.norm(r, &res));
		int stop;
		FS_TRY(g.diag(x, res, &stop));
		if (stop) {
			info->iters = iter + 1;
			info->status = FS_CONVERGED_USER;
			break;
		}
		if (res < tol) {
			info->iters = iter + 1;
			info->status = FS_CONVERGED_RTOL;
			break;
		}
		FS_TRY(g.check_finite(res));
		FS_TRY(g.P(r, z));
		rho0 = rho1;
		FS_TRY(g.dot(r, z, &rho1));
		const double beta = rho1 / rho0;
		FS_TRY(g.axpy(beta, p, z, p));
	}
	info->res_norm_final = (float)res;
	if (info->iters == 0)
		info->status = FS_DIVERGED_ITERS;
	return FS_OK;
}

// ----------------------------------------------------- flexible CG --
// cg.hh:145-244: one-step truncated flexible CG; the preconditioner may
// change between applications (a nested solver)
int gen_fcg(Gen &g, Vec *b, Vec *u, fs_solve_info *info) {
	const auto &set = g.s->set.base;
	Vec *r, *v, *w, *q, *d;
	FS_TRY(g.vec(0, &r));
	FS_TRY(g.vec(1, &v));
	FS_TRY(g.vec(2, &w));
	FS_TRY(g.vec(3, &q));
	FS_TRY(g.vec(4, &d));
	double b_norm;
	FS_TRY(g.norm(b, &b_norm));
	if (b_norm == 0.0)
		b_norm = 1.0;
	const double tol = set.rtol * b_norm;
	info->rhs_norm = (float)b_norm;
	if (set.use_zero_guess) {
		info->sol_norm_initial = 0;
		FS_TRY(fs_vec_set_scalar(hv(u), 0.0));
		FS_TRY(g.copy(b, r));
	}
	else {
		double un;
		FS_TRY(g.norm(u, &un));
		info->sol_norm_initial = (float)un;
		FS_TRY(g.residual(b, u, r));
	}
	double res;
	FS_TRY(g.norm(r, &res));
	info->res_norm_initial = (float)res;
	if (res < tol) {
		info->res_norm_final = (float)res;
		info->status = FS_CONVERGED_RTOL;
		return FS_OK;
	}
	double rho = 0;
	for (int iter = 0; iter < set.maxiter; ++iter) {
		FS_TRY(g.P(r, v));
		FS_TRY(g.A(v, w));
		double alpha, beta;
		FS_TRY(g.dot(v, r, &alpha));
		FS_TRY(g.dot(v, w, &beta));
		if (iter > 0) {
			double gamma;
			FS_TRY(g.dot(v, q, &gamma));
			FS_TRY(g.axpy((-gamma) / rho, d, v, d));
			FS_TRY(g.axpy((-gamma) / rho, q, w, q));
			rho = beta - (gamma * gamma) / rho;
		}
		else {
			FS_TRY(g.copy(v, d));
			FS_TRY(g.copy(w, q));
			rho = beta;
		}
		FS_TRY(g.axpy(alpha / rho, d, u, u));
		FS_TRY(g.axpy(-alpha / rho, q, r, r));
		FS_TRY(g.norm(r, &res));
		int stop;
		FS_TRY(g.diag(u, res, &stop));
		if (stop) {
			info->iters = iter + 1;
			info->status = FS_CONVERGED_USER;
			break;
		}
		if (res < tol) {
			info->iters = iter + 1;
			info->status = FS_CONVERGED_RTOL;
			break;
		}
		FS_TRY(g.check_finite(res));
	}
	info->res_norm_final = (float)res;
	if (info->iters == 0)
		info->status = FS_DIVERGED_ITERS;
	return FS_OK;
}

// ------------------------------------------------------- BiCGSTAB --
// bicgstab.hh:39-187, right preconditioned
int gen_bicgstab(Gen &g, Vec *b, Vec *x, fs_solve_info *info) {
	const auto &set = g.s->set.base;
	Vec *res, *rt, *p, *v, *ph, *sv, *sh, *t;
	FS_TRY(g.vec(0, &res));
	FS_TRY(g.vec(1, &rt));
	FS_TRY(g.vec(2, &p));
	FS_TRY(g.vec(3, &v));
	FS_TRY(g.vec(4, &ph));
	FS_TRY(g.vec(5, &sv));
	FS_TRY(g.vec(6, &sh));
	FS_TRY(g.vec(7, &t));
	double b_norm;
	FS_TRY(g.norm(b, &b_norm));
	if (b_norm == 0.)
		b_norm = 1.;
	const double tol = set.rtol * b_norm;
	info->rhs_norm = (float)b_norm;
	if (set.use_zero_guess) {
		info->sol_norm_initial = 0;
		FS_TRY(g.copy(b, res));
		FS_TRY(fs_vec_set_scalar(hv(x), 0.0));
	}
	else {
		double xn;
		FS_TRY(g.norm(x, &xn));
		info->sol_norm_initial = (float)xn;
		FS_TRY(g.residual(b, x, res));
	}
	double res_norm;
	FS_TRY(g.norm(res, &res_norm));
	double rt_norm = res_norm;
	info->res_norm_initial = (float)res_norm;
	if (res_norm < tol) {
		info->status = FS_CONVERGED_RTOL;
		info->res_norm_final = (float)res_norm;
		return FS_OK;
	}
	double alpha = 1.0, beta = 0.0, omega = 1.0;
	double rho[2] = {2.0, 1.0};
	FS_TRY(g.copy(res, rt));
	FS_TRY(fs_vec_set_scalar(hv(p), 0.0));
	FS_TRY(fs_vec_set_scalar(hv(v), 0.0));
	for (int iter = 0; iter < set.maxiter; ++iter) {
		FS_TRY(g.dot(rt, res, &rho[1]));
		const double angle = std::sqrt(std::fabs(rho[1]));
		if (angle < DBL_EPSILON * rt_norm) {
			// restart (bicgstab.hh:100-113): one loop index consumed
			FS_TRY(g.residual(b, x, res));
			FS_TRY(g.copy(res, rt));
			FS_TRY(g.norm(res, &res_norm));
			rho[1] = rt_norm = res_norm;
			FS_TRY(g.copy(res, p));
			++info->restarts;
			continue;
		}
		if (iter == 0)
			FS_TRY(g.copy(res, p));
		else {
			beta = (rho[1] / rho[0]) * (alpha / omega);
			FS_TRY(g.axpy(-omega, v, p, p));
			FS_TRY(g.axpy(beta, p, res, p));
		}
		FS_TRY(g.P(p, ph));
		FS_TRY(g.A(ph, v));
		FS_TRY(g.dot(rt, v, &alpha));
		if (!(alpha != 0.))
			return set_err(g.ctx, FS_ERR_BREAKDOWN, "BiCGSTAB: r~'v == 0 (bicgstab.hh:129)");
		alpha = rho[1] / alpha;
		FS_TRY(g.axpy(-alpha, v, res, sv));
		double s_norm;
		FS_TRY(g.norm(sv, &s_norm));
		if (s_norm < set.rtol) {
			// the unscaled early exit (bicgstab.hh:136-142)
			FS_TRY(g.axpy(alpha, ph, x, x));
			info->iters = iter;
			info->status = FS_CONVERGED_RTOL;
			break;
		}
		FS_TRY(g.P(sv, sh));
		FS_TRY(g.A(sh, t));
		double tt, ts;
		FS_TRY(g.dot(t, t, &tt));
		FS_TRY(g.dot(t, sv, &ts));
		omega = (tt == 0.0) ? 0.0 : ts / tt;
		FS_TRY(g.axpy(alpha, ph, x, x));
		FS_TRY(g.axpy(omega, sh, x, x));
		FS_TRY(g.axpy(-omega, t, sv, res));
		FS_TRY(g.norm(res, &res_norm));
		int stop;
		FS_TRY(g.diag(x, res_norm, &stop));
		if (stop) {
			info->status = FS_CONVERGED_USER;
			info->iters = iter + 1;
			break;
		}
		if (res_norm < tol) {
			info->status = FS_CONVERGED_RTOL;
			info->iters = iter + 1;
			break;
		}
		FS_TRY(g.check_finite(res_norm));
		if (omega == 0.0) {
			info->iters = iter + 1;
			info->status = FS_DIVERGED_BREAKDOWN;
			break;
		}
		rho[0] = rho[1];
	}
	info->res_norm_final = (float)res_norm;
	if (info->iters == 0)
		info->status = FS_DIVERGED_ITERS;
	return FS_OK;
}

// ---------------------------------------------------------- GMRES --
// gmres.hh:54-348: restarted GMRES with modified Gram-Schmidt, Givens
// rotations and back substitution on the host
struct Ls {
	int ld;
	std::vector<double> H, cs, sn, dw, dy;
	explicit Ls(int m)
		: ld(m + 1), H((size_t)(m + 1) * (m + 1), 0.0), cs(m + 1), sn(m + 1), dw(m + 1), dy(m + 1) {}
	double &h(int i, int j) { return H[(size_t)i + (size_t)ld * j]; }
	// gmres.hh:281-296
	void apply_givens(int i, int k) {
		const double x = h(i, k), y = h(i + 1, k), c = cs[i], s = sn[i];
		h(i, k) = c * x + s * y;
		h(i + 1, k) = -s * x + c * y;
	}
	// gmres.hh:298-331 (Bindel, Demmel, Kahan, Marques, Algorithm 1)
	void compute_givens(int k) {
		const double f = h(k, k), g = h(k + 1, k);
		double c, s;
		if (g == 0.0) {
			c = 1.0;
			s = 0.0;
		}
		else if (f == 0.0) {
			c = 0.0;
			s = (g < 0.0) ? -1.0 : 1.0;
		}
		else {
			const double r = 1.0 / std::sqrt(f * f + g * g);
			c = std::fabs(f) * r;
			s = std::copysign(g * r, f);
		}
		cs[k] = c;
		sn[k] = s;
	}
	// gmres.hh:333-348
	void back_solve(int nr) {
		dy[nr] = dw[nr] / h(nr, nr);
		for (int k = nr - 1; k >= 0; --k) {
			dy[k] = dw[k];
			for (int i = k + 1; i <= nr; ++i)
				dy[k] -= h(k, i) * dy[i];
			dy[k] = dy[k] / h(k, k);
		}
	}
};

int gen_gmres(Gen &g, Vec *b, Vec *x, fs_solve_info *info) {
	const fs_krylov_settings &S = g.s->set;
	const auto &set = S.base;
	const int mdim = S.max_krylov_dim < 0 ? set.maxiter : S.max_krylov_dim;
	const int max_dim = std::min(mdim, set.maxiter);
	const bool left = S.pre_side == FS_LEFT;
	Ls ls(std::max(1, max_dim));
	Vec *res, *z, *v;
	FS_TRY(g.vec(0, &res));
	FS_TRY(g.vec(1, &z));
	FS_TRY(g.vec(2, &v));
	std::vector<Vec *> V(ls.ld);
	for (int i = 0; i < ls.ld; ++i)
		FS_TRY(g.vec(3 + i, &V[i]));
	double b_norm;
	FS_TRY(g.norm(b, &b_norm));
	info->rhs_norm = (float)b_norm;
	if (b_norm < DBL_EPSILON)
		b_norm = 1.0;
	const double tol = set.rtol * b_norm;
	if (set.use_zero_guess)
		FS_TRY(fs_vec_set_scalar(hv(x), 0.0));
	auto start = [&](bool zero) -> int {
		if (left) {
			if (zero)
				FS_TRY(g.copy(b, V[0]));
			else
				FS_TRY(g.residual(b, x, V[0]));
			return g.P(V[0], res);
		}
		return zero ? g.copy(b, res) : g.residual(b, x, res);
	};
	FS_TRY(start(set.use_zero_guess != 0));
	double beta;
	FS_TRY(g.norm(res, &beta));
	info->res_norm_initial = (float)beta;
	if (beta < tol) {
		info->res_norm_final = (float)beta;
		info->status = FS_CONVERGED_RTOL;
		return FS_OK;
	}
	FS_TRY(fs_vec_scale_self(1.0 / beta, hv(res)));
	FS_TRY(g.copy(res, V[0]));
	ls.dw[0] = beta;
	double v_norm = beta;
	int k = 0;
	auto correct = [&](int nr) -> int {
		// gmres.hh:244-263
		ls.back_solve(nr);
		if (!left) {
			FS_TRY(fs_vec_set_scalar(hv(z), 0.0));
			for (int i = 0; i <= nr; ++i)
				FS_TRY(g.axpy(ls.dy[i], V[i], z, z));
			FS_TRY(g.P(z, v));
			return g.axpy(1.0, v, x, x);
		}
		for (int i = 0; i <= nr; ++i)
			FS_TRY(g.axpy(ls.dy[i], V[i], x, x));
		return FS_OK;
	};
	for (int iter = 0; iter < set.maxiter; ++iter) {
		if (!left) {
			FS_TRY(g.P(V[k], z));
			FS_TRY(g.A(z, v));
		}
		else {
			FS_TRY(g.A(V[k], z));
			FS_TRY(g.P(z, v));
		}
		// modified Gram-Schmidt, gmres.hh:265-279
		for (int j = 0; j <= k; ++j) {
			double hjk;
			FS_TRY(g.dot(v, V[j], &hjk));
			FS_TRY(g.axpy(-hjk, V[j], v, v));
			ls.h(j, k) = hjk;
		}
		FS_TRY(g.norm(v, &v_norm));
		ls.h(k + 1, k) = v_norm;
		if (v_norm != 0.0)
			FS_TRY(fs_vec_scale_self(1.0 / v_norm, hv(v)));
		FS_TRY(g.copy(v, V[k + 1]));
		for (int i = 0; i < k; ++i)
			ls.apply_givens(i, k);
		if (v_norm != 0.0) {
			ls.compute_givens(k);
			ls.apply_givens(k, k);
			ls.h(k + 1, k) = 0.0;
			const double xx = ls.dw[k], c = ls.cs[k], sn = ls.sn[k];
			ls.dw[k] = c * xx;
			ls.dw[k + 1] = -sn * xx;
		}
		v_norm = std::fabs(ls.dw[k + 1]);
		++k;
		int stop;
		FS_TRY(g.diag(x, v_norm, &stop));
		if (stop) {
			info->status = FS_CONVERGED_USER;
			info->iters = iter + 1;
			break;
		}
		if (v_norm < tol) {
			info->status = FS_CONVERGED_RTOL;
			info->iters = iter + 1;
			break;
		}
		FS_TRY(g.check_finite(v_norm));
		if (k == mdim && iter != set.maxiter - 1) {
			// restart (gmres.hh:208-225)
			FS_TRY(correct(k - 1));
			FS_TRY(start(false));
			double br;
			FS_TRY(g.norm(res, &br));
			FS_TRY(fs_vec_scale_self(1.0 / br, hv(res)));
			FS_TRY(g.copy(res, V[0]));
			ls.dw[0] = br;
			++info->restarts;
			k = 0;
		}
	}
	if (k > 0)
		FS_TRY(correct(k - 1));
	info->res_norm_final = (float)v_norm;
	if (info->iters == 0)
		info->status = FS_DIVERGED_ITERS;
	return FS_OK;
}

}  // namespace

bool needs_generic(const Solver *s) {
	if (s->method == FS_FCG || s->A->shell_fn)
		return true;
	return s->P.kind == FS_PRECOND_CSR || s->P.kind == FS_PRECOND_SOLVER;
}

int generic_apply(Solver *s, Vec *b, Vec *x, fs_solve_info *info) {
	Gen g(s);
	FS_TRY(g.setup());
	memset(info, 0, sizeof(*info));
	info->status = FS_STATUS_UNKNOWN;
	int st = FS_ERR_UNSUPPORTED;
	switch (s->method) {
	case FS_CG:
	case FS_CG_PIPELINED:  // with a general operator: the reference's CG loop
		st = gen_cg(g, b, x, info);
		break;
	case FS_FCG: st = gen_fcg(g, b, x, info); break;
	case FS_BICGSTAB: st = gen_bicgstab(g, b, x, info); break;
	case FS_GMRES: st = gen_gmres(g, b, x, info); break;
	default:
		st = set_err(s->ctx, FS_ERR_UNSUPPORTED,
		             "mixed-precision solvers take a stored or matrix-free operator and an "
		             "identity, Jacobi or diagonal preconditioner");
	}
	g.finish();
	if (st == FS_OK) {
		double xn;
		FS_TRY(fs_vec_l2norm(hv(x), &xn));
		info->sol_norm_final = (float)xn;
	}
	return st;
}

}  // namespace fsg
