/*
 * ORACLE -- test infrastructure only.  Nothing in the product links or calls
 * this file: it is the CPU checker that the tests, the smoke check and the
 * benchmark's CPU-baseline leg compare the CUDA path against.
 *
 * A plain-C restatement of flecsolve's serial Krylov path:
 *   - vec::seq_ops loops with left-to-right serial reductions
 *     (flecsolve/vectors/seq.hh:93-304),
 *   - mat::compressed_ops::spmv, the CSR row loop y_i = 0; y_i += a*x
 *     (flecsolve/matrices/seq.hh:177-193),
 *   - op::core::residual r = b - A x (flecsolve/operators/core.hh:129-142),
 *   - op::cg::apply (flecsolve/solvers/cg.hh:43-139),
 *   - op::fcg::apply, the flexible CG (flecsolve/solvers/cg.hh:145-244),
 *   - op::bicgstab::apply (flecsolve/solvers/bicgstab.hh:39-187),
 *   - op::gmres::apply / orthogonalize / Givens / back_solve / correct
 *     (flecsolve/solvers/gmres.hh:54-348),
 *   - mat::parcsr spmv split y = A_diag x + A_offd x_ghost
 *     (flecsolve/matrices/parcsr.hh:60-91).
 * Every floating-point operation is issued in the reference's order and
 * the file is compiled with -ffp-contract=off, so with the reference built
 * the same way the two agree bit for bit (checked by tests/test_oracle.py
 * against fixtures produced by the reference itself, tests/golden/).
 *
 * Scalars follow the reference types: tolerances are float
 * (solver_settings.hh:31-36) and the reported norms in solve_info are float
 * (solver_settings.hh:76-78).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define OR_API __attribute__((visibility("default")))

/* solve_info::stop_reason order, flecsolve/solvers/solver_settings.hh:64-72 */
enum {
	OR_CONVERGED_ATOL = 0,
	OR_CONVERGED_RTOL,
	OR_CONVERGED_USER,
	OR_DIVERGED_DTOL,
	OR_DIVERGED_ITERS,
	OR_DIVERGED_BREAKDOWN,
	OR_UNKNOWN,
	/* not a reference status: the reference aborts through flog_assert
	   (bicgstab.hh:129); the oracle reports it instead */
	OR_ASSERT_FAILED = 100
};

typedef struct {
	int maxiter;
	float rtol;
	float atol;
	int use_zero_guess;
} or_settings;

typedef struct {
	int status;
	int iters;
	int restarts;
	float res_norm_initial, res_norm_final;
	float sol_norm_initial, sol_norm_final;
	float rhs_norm;
} or_info;

/* CSR with 64-bit row offsets and 32-bit column ids */
typedef struct {
	int64_t nrows;
	const int64_t *rowptr;
	const int32_t *col;
	const double *val;
} or_csr;

/* diagnostic callable: returns nonzero to stop (converged_user) */
typedef int (*or_diag_fn)(void *user, const double *x, int64_t n, double res);

/* residual-norm history recorder, filled with the value handed to the
 * diagnostic each iteration (cg.hh:112, bicgstab.hh:160, gmres.hh:196) */
typedef struct {
	or_diag_fn fn;
	void *user;
	double *hist;
	int64_t cap;
	int64_t count;
} or_diag;

static int call_diag(or_diag *d, const double *x, int64_t n, double res) {
	if (!d)
		return 0;
	if (d->hist && d->count < d->cap)
		d->hist[d->count] = res;
	d->count++;
	return d->fn ? d->fn(d->user, x, n, res) : 0;
}

/* ------------------------------------------------------ vector ops --- */

/* Summation order of the reductions.  0 (default): the reference's serial
 * left-to-right loop.  The others exist only to measure how far a solver's
 * iteration count moves when the same sums are taken in another valid
 * order, as a parallel reduction takes them:
 *   1: blocks of 4096 products summed left to right, then the block sums
 *      left to right (a two-level reduction);
 *   2: right to left. */
static int dot_order = 0;
OR_API void or_set_dot_order(int order) { dot_order = order; }

/* Contraction switch (a checker option, default off): 1 fuses every
 * product into the sum or update it feeds -- the SpMV row sums, the dots and
 * the axpy updates -- as fma(a, b, c) with one rounding, the arithmetic of
 * the device's FMA kernels.  Off is the reference's separately rounded
 * products.  It measures how far an iteration count moves with that
 * rounding alone. */
static int contract = 0;
OR_API void or_set_contract(int on) { contract = on; }
#define OR_MAC(a, b, c) (contract ? fma((a), (b), (c)) : (a) * (b) + (c))

/* seq.hh:282-295, res += x_i * y_i left to right */
static double dot(int64_t n, const double *x, const double *y) {
	double res = 0.0;
	if (dot_order == 1) {
		for (int64_t b = 0; b < n; b += 4096) {
			const int64_t e = b + 4096 < n ? b + 4096 : n;
			double part = 0.0;
			for (int64_t i = b; i < e; ++i)
				part = OR_MAC(x[i], y[i], part);
			res += part;
		}
		return res;
	}
	if (dot_order == 2) {
		for (int64_t i = n - 1; i >= 0; --i)
			res = OR_MAC(x[i], y[i], res);
		return res;
	}
	for (int64_t i = 0; i < n; ++i)
		res = OR_MAC(x[i], y[i], res);
	return res;
}
/* seq.hh:221-247 with p = 2: sqrt(scalar_prod(x, x)) */
static double l2norm(int64_t n, const double *x) { return sqrt(dot(n, x, x)); }
/* seq.hh:171-174, z = alpha x + y */
static void axpy(int64_t n, double alpha, const double *x, const double *y,
                 double *z) {
	for (int64_t i = 0; i < n; ++i)
		z[i] = OR_MAC(alpha, x[i], y[i]);
}
static void copy(int64_t n, const double *s, double *d) {
	memcpy(d, s, (size_t)n * sizeof(double));
}
static void setv(int64_t n, double a, double *x) {
	for (int64_t i = 0; i < n; ++i)
		x[i] = a;
}
/* seq.hh:122-125, x_i *= alpha */
static void scale(int64_t n, double alpha, double *x) {
	for (int64_t i = 0; i < n; ++i)
		x[i] *= alpha;
}

/* ------------------------------------------------------- operators --- */

/* matrices/seq.hh:177-193 */
OR_API void or_spmv(const or_csr *A, const double *x, double *y) {
	for (int64_t i = 0; i < A->nrows; ++i) {
		y[i] = 0.;
		for (int64_t off = A->rowptr[i]; off < A->rowptr[i + 1]; ++off)
			y[i] = OR_MAC(A->val[off], x[A->col[off]], y[i]);
	}
}

/* preconditioner: NULL = op::I (copy, operators/shell.hh:94-95), otherwise a
 * CSR operator applied with the same row loop (the D^-1 test operator of
 * flecsolve/util/test/mesh.hh:123-140 is a 1-nnz-per-row CSR) */
static void papply(const or_csr *P, int64_t n, const double *x, double *y) {
	if (P)
		or_spmv(P, x, y);
	else
		copy(n, x, y);
}

/* operators/core.hh:135-142: apply(x, r); r = b - r */
static void residual(const or_csr *A, const double *b, const double *x,
                     double *r) {
	or_spmv(A, x, r);
	for (int64_t i = 0; i < A->nrows; ++i)
		r[i] = b[i] - r[i];
}

OR_API void or_residual(const or_csr *A, const double *b, const double *x,
                        double *r) {
	residual(A, b, x, r);
}

/* D^-1 as in flecsolve/util/test/mesh.hh:123-140: values 1.0 / a_ii */
OR_API void or_diag_inv(const or_csr *A, double *dinv) {
	for (int64_t i = 0; i < A->nrows; ++i) {
		dinv[i] = 0.0;
		for (int64_t off = A->rowptr[i]; off < A->rowptr[i + 1]; ++off)
			if (A->col[off] == i)
				dinv[i] = 1.0 / A->val[off];
	}
}

OR_API double or_dot(int64_t n, const double *x, const double *y) {
	return dot(n, x, y);
}

/* ------------------------------------------------------------- CG --- */

/* flecsolve/solvers/cg.hh:43-139 */
OR_API int or_cg(const or_settings *s, const or_csr *A, const or_csr *P,
                 const double *b, double *x, or_diag *diag, or_info *info) {
	int64_t n = A->nrows;
	memset(info, 0, sizeof(*info));
	info->status = OR_UNKNOWN;
	info->res_norm_initial = NAN; /* indeterminate in the reference */
	double *r = malloc(n * sizeof(double)), *z = malloc(n * sizeof(double));
	double *p = malloc(n * sizeof(double)), *w = malloc(n * sizeof(double));

	double b_norm = l2norm(n, b);
	if (b_norm == 0.0)
		b_norm = 1.0;
	const double terminate_tol = s->rtol * b_norm;
	info->rhs_norm = (float)b_norm;

	if (s->use_zero_guess) {
		info->sol_norm_initial = 0;
		setv(n, 0., x);
		copy(n, b, r);
	}
	else {
		info->sol_norm_initial = (float)l2norm(n, x);
		residual(A, b, x, r);
	}

	double current_res = l2norm(n, r);
	if (current_res < terminate_tol) {
		info->res_norm_initial = (float)current_res;
		info->res_norm_final = (float)current_res;
		info->status = OR_CONVERGED_RTOL;
		goto done;
	}

	papply(P, n, r, z);
	double rho[2] = {2.0, 0.0};
	rho[1] = dot(n, z, r);
	rho[0] = rho[1];
	copy(n, z, p);
	for (int iter = 0; iter < s->maxiter; iter++) {
		double beta = 1.0;
		or_spmv(A, p, w);
		double alpha = dot(n, w, p);
		alpha = rho[1] / alpha;
		axpy(n, alpha, p, x, x);
		axpy(n, -alpha, w, r, r);
		current_res = l2norm(n, r);
		if (call_diag(diag, x, n, current_res)) {
			info->iters = iter + 1;
			info->status = OR_CONVERGED_USER;
			break;
		}
		if (current_res < terminate_tol) {
			info->iters = iter + 1;
			info->status = OR_CONVERGED_RTOL;
			break;
		}
		papply(P, n, r, z);
		rho[0] = rho[1];
		rho[1] = dot(n, r, z);
		beta = rho[1] / rho[0];
		axpy(n, beta, p, z, p);
	}
	info->res_norm_final = (float)current_res;
	info->sol_norm_final = (float)l2norm(n, x);
	if (info->iters == 0)
		info->status = OR_DIVERGED_ITERS;
done:
	free(r);
	free(z);
	free(p);
	free(w);
	return info->status;
}

/* ---------------------------------------------------- flexible CG --- */

/* The preconditioner of or_fcg: P itself, or (inner_iters > 0) that many
 * iterations of Jacobi-PCG on A with P as its preconditioner, from a zero
 * guess, rtol 0 (a nested cg::solver bound as the preconditioner, the
 * solvers/test/nka.cc:72-80 pattern) */
typedef struct {
	const or_csr *A, *P;
	int inner_iters;
} fcg_pc;

static void fcg_papply(const fcg_pc *pc, int64_t n, const double *r, double *z) {
	if (pc->inner_iters <= 0) {
		papply(pc->P, n, r, z);
		return;
	}
	or_settings s = {pc->inner_iters, 0.f, 0.f, 1};
	or_info info;
	or_cg(&s, pc->A, pc->P, r, z, NULL, &info);
}

/* flecsolve/solvers/cg.hh:145-244 */
OR_API int or_fcg(const or_settings *s, const or_csr *A, const or_csr *P, int inner_iters,
                  const double *b, double *u, or_diag *diag, or_info *info) {
	int64_t n = A->nrows;
	memset(info, 0, sizeof(*info));
	info->status = OR_UNKNOWN;
	info->res_norm_initial = NAN; /* indeterminate in the reference */
	fcg_pc pc = {A, P, inner_iters};
	double *wk = malloc(5 * n * sizeof(double));
	double *r = wk, *v = wk + n, *w = wk + 2 * n, *q = wk + 3 * n, *d = wk + 4 * n;

	double b_norm = l2norm(n, b);
	if (b_norm == 0.0)
		b_norm = 1.0;
	const double terminate_tol = s->rtol * b_norm;
	info->rhs_norm = (float)b_norm;
	if (s->use_zero_guess) {
		info->sol_norm_initial = 0;
		setv(n, 0., u);
		copy(n, b, r);
	}
	else {
		info->sol_norm_initial = (float)l2norm(n, u);
		residual(A, b, u, r);
	}
	double current_res = l2norm(n, r);
	if (current_res < terminate_tol) {
		info->res_norm_initial = (float)current_res;
		info->res_norm_final = (float)current_res;
		info->status = OR_CONVERGED_RTOL;
		goto done;
	}
	double rho = 0;
	for (int iter = 0; iter < s->maxiter; iter++) {
		fcg_papply(&pc, n, r, v);
		or_spmv(A, v, w);
		double alpha = dot(n, v, r);
		double beta = dot(n, v, w);
		if (iter > 0) {
			double gamma = dot(n, v, q);
			axpy(n, (-gamma) / rho, d, v, d);
			axpy(n, (-gamma) / rho, q, w, q);
			rho = beta - (gamma * gamma) / rho;
		}
		else {
			copy(n, v, d);
			copy(n, w, q);
			rho = beta;
		}
		axpy(n, alpha / rho, d, u, u);
		axpy(n, -alpha / rho, q, r, r);
		current_res = l2norm(n, r);
		if (call_diag(diag, u, n, current_res)) {
			info->iters = iter + 1;
			info->status = OR_CONVERGED_USER;
			break;
		}
		if (current_res < terminate_tol) {
			info->iters = iter + 1;
			info->status = OR_CONVERGED_RTOL;
			break;
		}
	}
	info->res_norm_final = (float)current_res;
	info->sol_norm_final = (float)l2norm(n, u);
	if (info->iters == 0)
		info->status = OR_DIVERGED_ITERS;
done:
	free(wk);
	return info->status;
}

/* ------------------------------------------------------- BiCGSTAB --- */

/* flecsolve/solvers/bicgstab.hh:39-187 */
OR_API int or_bicgstab(const or_settings *s, const or_csr *A, const or_csr *P,
                       const double *b, double *x, or_diag *diag,
                       or_info *info) {
	int64_t n = A->nrows;
	memset(info, 0, sizeof(*info));
	info->status = OR_UNKNOWN;
	double *wk = malloc(8 * n * sizeof(double));
	double *res = wk, *r_tilde = wk + n, *p = wk + 2 * n, *v = wk + 3 * n;
	double *p_hat = wk + 4 * n, *sv = wk + 5 * n, *s_hat = wk + 6 * n,
	       *t = wk + 7 * n;

	double b_norm = l2norm(n, b);
	if (b_norm == 0.)
		b_norm = 1.;
	const double terminate_tol = s->rtol * b_norm;
	info->rhs_norm = (float)b_norm;

	if (s->use_zero_guess) {
		info->sol_norm_initial = 0;
		copy(n, b, res);
		setv(n, 0., x);
	}
	else {
		info->sol_norm_initial = (float)l2norm(n, x);
		residual(A, b, x, res);
	}

	double res_norm = l2norm(n, res);
	double r_tilde_norm = res_norm;
	info->res_norm_initial = (float)res_norm;
	if (res_norm < terminate_tol) {
		info->status = OR_CONVERGED_RTOL;
		info->res_norm_initial = (float)res_norm;
		info->res_norm_final = (float)res_norm;
		goto done;
	}

	double alpha = 1.0, beta = 0.0, omega = 1.0;
	double rho[2] = {2.0, 1.0}; /* std::vector<real>{2, 1.0} */
	copy(n, res, r_tilde);
	setv(n, 0., p);
	setv(n, 0., v);
	for (int iter = 0; iter < s->maxiter; iter++) {
		rho[1] = dot(n, r_tilde, res);
		double angle = sqrt(fabs(rho[1]));
		double eps = DBL_EPSILON;
		if (angle < eps * r_tilde_norm) {
			residual(A, b, x, res);
			copy(n, res, r_tilde);
			res_norm = l2norm(n, res);
			rho[1] = r_tilde_norm = res_norm;
			copy(n, res, p);
			++info->restarts;
			continue;
		}
		if (iter == 0) {
			copy(n, res, p);
		}
		else {
			beta = (rho[1] / rho[0]) * (alpha / omega);
			axpy(n, -omega, v, p, p);
			axpy(n, beta, p, res, p);
		}
		papply(P, n, p, p_hat);
		or_spmv(A, p_hat, v);
		alpha = dot(n, r_tilde, v);
		if (!(alpha != 0.)) {
			info->status = OR_ASSERT_FAILED; /* flog_assert, bicgstab.hh:129 */
			goto done;
		}
		alpha = rho[1] / alpha;
		axpy(n, -alpha, v, res, sv);
		const double s_norm = l2norm(n, sv);
		if (s_norm < s->rtol) {
			axpy(n, alpha, p_hat, x, x);
			info->iters = iter;
			info->status = OR_CONVERGED_RTOL;
			break;
		}
		papply(P, n, sv, s_hat);
		or_spmv(A, s_hat, t);
		double t_sqnorm = dot(n, t, t);
		double t_dot_s = dot(n, t, sv);
		omega = (t_sqnorm == 0.0) ? 0.0 : t_dot_s / t_sqnorm;
		axpy(n, alpha, p_hat, x, x);
		axpy(n, omega, s_hat, x, x);
		axpy(n, -omega, t, sv, res);
		res_norm = l2norm(n, res);
		if (call_diag(diag, x, n, res_norm)) {
			info->status = OR_CONVERGED_USER;
			info->iters = iter + 1;
			break;
		}
		if (res_norm < terminate_tol) {
			info->status = OR_CONVERGED_RTOL;
			info->iters = iter + 1;
			break;
		}
		if (omega == 0.0) {
			info->iters = iter + 1;
			info->status = OR_DIVERGED_BREAKDOWN;
			break;
		}
		rho[0] = rho[1];
	}
	info->res_norm_final = (float)res_norm;
	info->sol_norm_final = (float)l2norm(n, x);
	if (info->iters == 0)
		info->status = OR_DIVERGED_ITERS;
done:
	free(wk);
	return info->status;
}

/* ---------------------------------------------------------- GMRES --- */

enum { OR_LEFT = 0, OR_RIGHT = 1 };

typedef struct {
	or_settings base;
	int max_krylov_dim;
	int pre_side;
	int restart;
} or_gmres_settings;

#define KRYLOV_DIM_BOUND 100 /* gmres.hh:31 */

typedef struct {
	int64_t n;
	int ld; /* max_dim + 1, column-major leading dimension (gmres.hh:60-65) */
	double *H, *cs, *sn, *dw, *dy;
	double **basis;
} gm_state;

#define HM(g, i, j) ((g)->H[(size_t)(i) + (size_t)(g)->ld * (size_t)(j)])

/* gmres.hh:265-279, modified Gram-Schmidt */
static void orthogonalize(gm_state *g, double *v, int k) {
	for (int j = 0; j < k; j++) {
		const double h_jk = dot(g->n, v, g->basis[j]);
		axpy(g->n, -h_jk, g->basis[j], v, v);
		HM(g, j, k - 1) = h_jk;
	}
	const double v_norm = l2norm(g->n, v);
	HM(g, k, k - 1) = v_norm;
}

/* gmres.hh:281-296 */
static void apply_givens(gm_state *g, int i, int k) {
	double x = HM(g, i, k), y = HM(g, i + 1, k);
	double c = g->cs[i], s = g->sn[i];
	HM(g, i, k) = c * x + s * y;
	HM(g, i + 1, k) = -s * x + c * y;
}

/* gmres.hh:298-331 (Bindel, Demmel, Kahan, Marques, Algorithm 1) */
static void compute_givens(gm_state *g, int k) {
	double f = HM(g, k, k), gg = HM(g, k + 1, k);
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

/* gmres.hh:333-348 */
static void back_solve(gm_state *g, int nr) {
	g->dy[nr] = g->dw[nr] / HM(g, nr, nr);
	for (int k = nr - 1; k >= 0; k--) {
		g->dy[k] = g->dw[k];
		for (int i = k + 1; i <= nr; i++)
			g->dy[k] -= HM(g, k, i) * g->dy[i];
		g->dy[k] = g->dy[k] / HM(g, k, k);
	}
}

/* gmres.hh:244-263 */
static void correct(gm_state *g, int side, int nr, const or_csr *P, double *z,
                    double *v, double *x) {
	if (side == OR_RIGHT) {
		setv(g->n, 0.0, z);
		for (int i = 0; i <= nr; i++)
			axpy(g->n, g->dy[i], g->basis[i], z, z);
		papply(P, g->n, z, v);
		axpy(g->n, 1.0, v, x, x);
	}
	else {
		for (int i = 0; i <= nr; i++)
			axpy(g->n, g->dy[i], g->basis[i], x, x);
	}
}

/* settings::validate, gmres.hh:394-404; returns 0 when the reference would
 * pass its assertions */
OR_API int or_gmres_validate(or_gmres_settings *s) {
	if (s->max_krylov_dim < 0)
		s->max_krylov_dim = s->base.maxiter;
	if (s->max_krylov_dim > KRYLOV_DIM_BOUND)
		return -1;
	if (!s->restart && s->base.maxiter > s->max_krylov_dim)
		return -2;
	return 0;
}

/* flecsolve/solvers/gmres.hh:54-241 */
OR_API int or_gmres(or_gmres_settings *s, const or_csr *A, const or_csr *P,
                    const double *b, double *x, or_diag *diag, or_info *info) {
	int64_t n = A->nrows;
	memset(info, 0, sizeof(*info));
	info->status = OR_UNKNOWN;
	if (or_gmres_validate(s)) {
		info->status = OR_ASSERT_FAILED;
		return info->status;
	}
	int max_dim = s->max_krylov_dim < s->base.maxiter ? s->max_krylov_dim
	                                                  : s->base.maxiter;
	gm_state g;
	g.n = n;
	g.ld = max_dim + 1;
	g.H = calloc((size_t)g.ld * g.ld, sizeof(double));
	g.cs = calloc(g.ld, sizeof(double));
	g.sn = calloc(g.ld, sizeof(double));
	g.dw = calloc(g.ld, sizeof(double));
	g.dy = calloc(g.ld, sizeof(double));
	g.basis = malloc(g.ld * sizeof(double *));
	double *store = malloc((size_t)(g.ld + 3) * n * sizeof(double));
	double *res = store, *z = store + n, *v = store + 2 * n;
	for (int i = 0; i < g.ld; ++i)
		g.basis[i] = store + (size_t)(3 + i) * n;

	double b_norm = l2norm(n, b);
	info->rhs_norm = (float)b_norm;
	if (b_norm < DBL_EPSILON)
		b_norm = 1.0;
	const double terminate_tol = s->base.rtol * b_norm;
	if (s->base.use_zero_guess)
		setv(n, 0., x);
	if (s->pre_side == OR_LEFT) {
		if (s->base.use_zero_guess)
			copy(n, b, g.basis[0]);
		else
			residual(A, b, x, g.basis[0]);
		papply(P, n, g.basis[0], res);
	}
	else {
		if (s->base.use_zero_guess)
			copy(n, b, res);
		else
			residual(A, b, x, res);
	}
	const double beta = l2norm(n, res);
	info->res_norm_initial = (float)beta;
	if (beta < terminate_tol) {
		info->res_norm_final = (float)beta;
		info->status = OR_CONVERGED_RTOL;
		goto done;
	}
	scale(n, 1.0 / beta, res);
	copy(n, res, g.basis[0]);
	g.dw[0] = beta;
	double v_norm = beta;
	int k = 0;
	for (int iter = 0; iter < s->base.maxiter; iter++) {
		if (s->pre_side == OR_RIGHT) {
			papply(P, n, g.basis[k], z);
			or_spmv(A, z, v);
		}
		else {
			or_spmv(A, g.basis[k], z);
			papply(P, n, z, v);
		}
		orthogonalize(&g, v, k + 1);
		v_norm = HM(&g, k + 1, k);
		if (v_norm != 0.0)
			scale(n, 1.0 / v_norm, v);
		copy(n, v, g.basis[k + 1]);
		for (int i = 0; i < k; i++)
			apply_givens(&g, i, k);
		if (v_norm != 0.0) {
			compute_givens(&g, k);
			apply_givens(&g, k, k);
			HM(&g, k + 1, k) = 0.0;
			double xx = g.dw[k], c = g.cs[k], sn = g.sn[k];
			g.dw[k] = c * xx;
			g.dw[k + 1] = -sn * xx;
		}
		v_norm = fabs(g.dw[k + 1]);
		++k;
		if (call_diag(diag, x, n, v_norm)) {
			info->status = OR_CONVERGED_USER;
			info->iters = iter + 1;
			break;
		}
		if (v_norm < terminate_tol) {
			info->status = OR_CONVERGED_RTOL;
			info->iters = iter + 1;
			break;
		}
		if (k == s->max_krylov_dim && iter != s->base.maxiter - 1) {
			back_solve(&g, k - 1);
			correct(&g, s->pre_side, k - 1, P, z, v, x);
			if (s->pre_side == OR_LEFT) {
				residual(A, b, x, g.basis[0]);
				papply(P, n, g.basis[0], res);
			}
			else
				residual(A, b, x, res);
			const double betar = l2norm(n, res);
			scale(n, 1.0 / betar, res);
			copy(n, res, g.basis[0]);
			g.dw[0] = betar;
			++info->restarts;
			k = 0;
		}
	}
	if (k > 0) {
		back_solve(&g, k - 1);
		correct(&g, s->pre_side, k - 1, P, z, v, x);
	}
	info->res_norm_final = (float)v_norm;
	info->sol_norm_final = (float)l2norm(n, x);
	if (info->iters == 0)
		info->status = OR_DIVERGED_ITERS;
done:
	free(g.H);
	free(g.cs);
	free(g.sn);
	free(g.dw);
	free(g.dy);
	free(g.basis);
	free(store);
	return info->status;
}

/* ------------------------------------------------ parallel CSR SpMV --- */

/* The first row of colour c when N rows are split into `parts` colours as
 * flecsi::util::equal_map splits them (FleCSI 2.4, flecsi/util/color_map.hh,
 * a dependency absent from the reference; its published rule restated here):
 * blocks of q = N / parts rows, the first r = N % parts of them one row
 * longer, so block c starts at c q + min(c, r). */
static int64_t or_equal_map_start(int64_t N, int parts, int64_t c) {
	const int64_t q = N / parts, r = N % parts;
	return c * q + (c < r ? c : r);
}

/* mat::parcsr spmv over a row-block partition into `parts` colours
 * (flecsolve/matrices/parcsr.hh:60-91, 146-156, topo/csr.hh:482-618): for
 * every row the owned-column entries (diag block) and the ghost-column
 * entries (offd block) are summed separately, each left to right in CSR
 * order, and then y = y_diag + y_offd (the y.add(y, tmp) of parcsr.hh:67).
 * Row blocks are the equal_map blocks above (parcsr.hh:149-151). */
OR_API void or_parcsr_spmv(const or_csr *A, int parts, const double *x,
                           double *y) {
	int64_t N = A->nrows;
	for (int c = 0; c < parts; ++c) {
		int64_t r0 = or_equal_map_start(N, parts, c);
		int64_t r1 = or_equal_map_start(N, parts, c + 1);
		for (int64_t i = r0; i < r1; ++i) {
			double yd = 0., yo = 0.;
			for (int64_t off = A->rowptr[i]; off < A->rowptr[i + 1]; ++off) {
				int64_t j = A->col[off];
				if (j >= r0 && j < r1)
					yd += A->val[off] * x[j];
				else
					yo += A->val[off] * x[j];
			}
			y[i] = yd + yo;
		}
	}
}
