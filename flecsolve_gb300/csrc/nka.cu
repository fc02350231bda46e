// NKA: the nonlinear Krylov accelerator of Carlson and Miller (SIAM J. Sci.
// Comput. 19, 1998), as flecsolve's op::nka runs it (flecsolve/solvers/
// nka.hh:31-605), over device vectors.
//
// The outer loop, the acceleration subspace and its small normal-equation
// factorisation are host work (a few scalars per iteration); every vector
// operation -- the residual, the preconditioner solve, the dots with the
// subspace vectors, the corrections -- runs on the device through the
// library's vector operations, CSR operator and bound Krylov solvers.  The
// preconditioner is a bound solver (the reference's solvers/test/nka.cc:72-80
// uses a CG solver as P) applied as P.apply(res, correction), or none.
//
// Subspace (nka.hh:236-335): the corrections v_k and the function
// differences w_k of earlier iterations, kept as an ordered list, newest
// first, in (max_dim + 1) slots each.  h[a][b], for slots a newer than b,
// holds w_a . w_b (the normal matrix, implicit unit diagonal); h[b][a] the
// Cholesky factor of it and h[a][a] the factor's diagonal.  A vector whose
// factor diagonal falls to angle_tol or below is dropped; past max_dim the
// oldest is dropped.
#include <cmath>
#include <cstring>
#include <vector>

#include "solver.cuh"

namespace fsg {

namespace {

constexpr int kMagicNka = 0x46534E4B;  // 'FSNK'
constexpr int kNkaMaxDim = 64;

struct Nka {
	int magic = kMagicNka;
	Ctx *ctx = nullptr;
	fs_nka_settings set{};
	Csr *F = nullptr;
	fs_residual_fn fres = nullptr;
	void *fres_user = nullptr;
	Solver *P = nullptr;
	fs_diag_fn diag = nullptr;
	void *diag_user = nullptr;
	int64_t n = 0;
	Vec *sol = nullptr, *res = nullptr, *cor = nullptr;
	std::vector<Vec *> w, v;        // max_dim + 1 slots each
	// acceleration subspace: slots in use, newest first; free slots
	std::vector<int> order, free_slots;
	std::vector<double> h;          // (max_dim + 1)^2, h[a * ld + b]
	int ld = 0;
	bool have_subspace = false, have_pending = false;
	int current_correction = 0;

	double &H(int a, int b) { return h[(size_t)a * ld + b]; }
};

bool ok_nka(const Nka *k) { return k && k->magic == kMagicNka && ok_ctx(k->ctx); }

fs_vec hv(Vec *v) { return reinterpret_cast<fs_vec>(v); }

int vdot(Vec *a, Vec *b, double *out) { return fs_vec_dot(hv(a), hv(b), out); }

// settings::validate (nka.hh:518-526); the assertion sites return
// FS_ERR_BREAKDOWN, as the library's other flog_assert sites do
int validate(Ctx *ctx, const fs_nka_settings &s) {
	if (s.adaptive_damping && !s.use_damping)
		return set_err(ctx, FS_ERR_BREAKDOWN, "NKA: damping must be enabled for adaptive_damping");
	if (s.max_dim <= 0)
		return set_err(ctx, FS_ERR_BREAKDOWN, "NKA: maximum dimension must be > 0.");
	if (!(s.angle_tol > 0.))
		return set_err(ctx, FS_ERR_BREAKDOWN, "NKA: angle tolerance must be > 0.0.");
	if (s.max_dim > kNkaMaxDim)
		return set_err(ctx, FS_ERR_UNSUPPORTED, "NKA: max_dim above %d", kNkaMaxDim);
	if (s.use_qr)
		return set_err(ctx, FS_ERR_UNSUPPORTED, "NKA: QR factorization not implemented");
	return FS_OK;
}

// the empty subspace (nka.hh:50-63)
void reset_subspace(Nka *k) {
	k->order.clear();
	k->free_slots.clear();
	for (int s = k->set.max_dim; s >= 0; --s)
		k->free_slots.push_back(s);  // slot 0 is handed out first
	std::fill(k->h.begin(), k->h.end(), 0.0);
	k->have_subspace = false;
	k->have_pending = false;
	k->current_correction = 0;
}

void drop_at(Nka *k, size_t pos) {
	k->free_slots.push_back(k->order[pos]);
	k->order.erase(k->order.begin() + (long)pos);
}

// relax (nka.hh:140-146): forget the pending difference
void relax(Nka *k) {
	if (k->have_pending) {
		drop_at(k, 0);
		k->have_pending = false;
	}
}

// Cholesky factorisation of the normal matrix W^T W along the list, newest
// first, dropping vectors that nearly lie in the span of the newer ones
// (nka.hh:148-203)
void factorize(Nka *k) {
	const double tol2 = k->set.angle_tol * k->set.angle_tol;
	k->H(k->order[0], k->order[0]) = 1.0;
	int nvec = 1;
	for (size_t pk = 1; pk < k->order.size();) {
		++nvec;
		const int sk = k->order[pk];
		if (nvec > k->set.max_dim) {
			// the newest max_dim vectors fill the subspace: drop the oldest
			drop_at(k, k->order.size() - 1);
			break;
		}
		double hkk = 1.0;
		for (size_t pj = 0; pj < pk; ++pj) {
			const int sj = k->order[pj];
			double hkj = k->H(sj, sk);
			for (size_t pi = 0; pi < pj; ++pi) {
				const int si = k->order[pi];
				hkj -= k->H(sk, si) * k->H(sj, si);
			}
			hkj /= k->H(sj, sj);
			k->H(sk, sj) = hkj;
			hkk -= hkj * hkj;
		}
		if (hkk > tol2) {
			k->H(sk, sk) = std::sqrt(hkk);
			++pk;
		}
		else {
			drop_at(k, pk);  // the next vector moves into position pk
			--nvec;
		}
	}
}

// Coefficients of f's projection on the span of the w's (nka.hh:205-234):
// forward substitution newest to oldest, backward oldest to newest
int project(Nka *k, Vec *f, std::vector<double> &cv) {
	cv.assign((size_t)k->set.max_dim + 1, 0.0);
	const size_t m = k->order.size();
	for (size_t pj = 0; pj < m; ++pj) {
		const int sj = k->order[pj];
		double cj;
		FS_TRY(vdot(f, k->w[(size_t)sj], &cj));
		for (size_t pi = 0; pi < pj; ++pi) {
			const int si = k->order[pi];
			cj -= k->H(sj, si) * cv[(size_t)si];
		}
		cv[(size_t)sj] = cj / k->H(sj, sj);
	}
	for (size_t rj = m; rj-- > 0;) {
		const int sj = k->order[rj];
		double cj = cv[(size_t)sj];
		for (size_t ri = m - 1; ri > rj; --ri) {
			const int si = k->order[ri];
			cj -= k->H(si, sj) * cv[(size_t)si];
		}
		cv[(size_t)sj] = cj / k->H(sj, sj);
	}
	return FS_OK;
}

// The accelerated correction from the preconditioned residual f, in place
// (nka.hh:236-335)
int compute_correction(Nka *k, Vec *f) {
	++k->current_correction;
	if (k->have_pending) {
		const int s1 = k->order[0];
		Vec *w1 = k->w[(size_t)s1], *v1 = k->v[(size_t)s1];
		// the newest function difference w_1 = w_1 - f
		FS_TRY(fs_vec_axpy(-1.0, hv(f), hv(w1), hv(w1)));
		double s;
		FS_TRY(fs_vec_l2norm(hv(w1), &s));
		if (s == 0.0) {
			// no information in this difference: forget it (the reference
			// warns and relaxes, then goes on to scale by 1/0)
			relax(k);
		}
		else {
			FS_TRY(fs_vec_scale_self(1.0 / s, hv(w1)));
			FS_TRY(fs_vec_scale_self(1.0 / s, hv(v1)));
			for (size_t p = 1; p < k->order.size(); ++p) {
				double d;
				FS_TRY(vdot(w1, k->w[(size_t)k->order[p]], &d));
				k->H(s1, k->order[p]) = d;
			}
			factorize(k);
			k->have_subspace = true;
			k->have_pending = false;
		}
	}
	if (k->free_slots.empty())
		return set_err(k->ctx, FS_ERR_BREAKDOWN, "NKA: free list error");
	const int loc = k->free_slots.back();
	k->free_slots.pop_back();
	// keep f to turn it into the next difference
	FS_TRY(fs_vec_copy(hv(f), hv(k->w[(size_t)loc])));
	if (k->have_subspace) {
		std::vector<double> cv;
		FS_TRY(project(k, f, cv));
		for (int s : k->order) {
			FS_TRY(fs_vec_axpy(cv[(size_t)s], hv(k->v[(size_t)s]), hv(f), hv(f)));
			FS_TRY(fs_vec_axpy(-cv[(size_t)s], hv(k->w[(size_t)s]), hv(f), hv(f)));
		}
		if (k->set.use_damping) {
			double eta = k->set.damping_factor;
			if (k->set.adaptive_damping)
				eta = 1.0 - std::pow(0.9, std::min(k->current_correction, k->set.max_dim));
			FS_TRY(fs_vec_scale_self(eta, hv(f)));
		}
	}
	// the correction, accelerated or not, for the next call
	FS_TRY(fs_vec_copy(hv(f), hv(k->v[(size_t)loc])));
	k->order.insert(k->order.begin(), loc);
	k->have_pending = true;
	return FS_OK;
}

// res = F(u) - f: the operator's residual f - F(u), negated (nka.hh:86-87)
int neg_residual(Nka *k, Vec *f, Vec *u, Vec *res) {
	if (k->fres) {
		const int st = k->fres(k->fres_user, hv(f), hv(u), hv(res));
		if (st != FS_OK)
			return set_err(k->ctx, st, "NKA: residual callback returned %d", st);
	}
	else
		FS_TRY(fs_csr_residual(reinterpret_cast<fs_csr>(k->F), hv(f), hv(u), hv(res)));
	return fs_vec_scale_self(-1.0, hv(res));
}

}  // namespace

}  // namespace fsg

using namespace fsg;

extern "C" {

FS_API int fs_nka_settings_default(fs_nka_settings *s) {
	if (!s)
		return FS_ERR_INVALID_ARG;
	std::memset(s, 0, sizeof(*s));
	// solver_options defaults (solver_settings.hh:40-52) and nka::options
	// (nka.hh:536-552); max_dim has no default there (required)
	s->base.maxiter = 100;
	s->max_dim = 0;
	s->angle_tol = 0.9;
	s->freeze_pc = 1;
	s->damping_factor = 1.0;
	return FS_OK;
}

FS_API int fs_nka_create(fs_ctx ch, const fs_nka_settings *s, fs_csr Fh, fs_residual_fn fres,
                         void *fres_user, fs_solver Ph, fs_nka *out) {
	Ctx *ctx = reinterpret_cast<Ctx *>(ch);
	Csr *F = reinterpret_cast<Csr *>(Fh);
	Solver *P = reinterpret_cast<Solver *>(Ph);
	if (!ok_ctx(ctx) || !s || !out)
		return FS_ERR_BAD_HANDLE;
	*out = nullptr;
	if (!F && !fres)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_nka_create: an operator or a residual is required");
	if (F && !ok_csr(F))
		return FS_ERR_BAD_HANDLE;
	if (Ph && !ok_slv(P))
		return FS_ERR_BAD_HANDLE;
	FS_TRY(validate(ctx, *s));
	int64_t n = F ? F->nrows : (P ? P->n : -1);
	if (n < 0)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_nka_create: the size comes from F or P");
	if ((F && F->nrows != F->ncols) || (P && P->n != n))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_nka_create: F and P sizes differ");
	Nka *k = new Nka();
	k->ctx = ctx;
	k->set = *s;
	k->F = F;
	k->fres = fres;
	k->fres_user = fres_user;
	k->P = P;
	k->n = n;
	const int slots = s->max_dim + 1;
	k->ld = slots;
	k->h.assign((size_t)slots * slots, 0.0);
	auto mk = [&](Vec **v) {
		return fs_vec_create(ch, n, FS_F64, reinterpret_cast<fs_vec *>(v));
	};
	int st = mk(&k->sol);
	if (st == FS_OK)
		st = mk(&k->res);
	if (st == FS_OK)
		st = mk(&k->cor);
	k->w.assign((size_t)slots, nullptr);
	k->v.assign((size_t)slots, nullptr);
	for (int i = 0; i < slots && st == FS_OK; ++i) {
		st = mk(&k->w[(size_t)i]);
		if (st == FS_OK)
			st = mk(&k->v[(size_t)i]);
	}
	if (st != FS_OK) {
		fs_nka_destroy(reinterpret_cast<fs_nka>(k));
		return st;
	}
	reset_subspace(k);
	*out = reinterpret_cast<fs_nka>(k);
	return FS_OK;
}

FS_API int fs_nka_set_diagnostic(fs_nka h, fs_diag_fn fn, void *user) {
	Nka *k = reinterpret_cast<Nka *>(h);
	if (!ok_nka(k))
		return FS_ERR_BAD_HANDLE;
	k->diag = fn;
	k->diag_user = user;
	return FS_OK;
}

FS_API int fs_nka_reset(fs_nka h) {
	Nka *k = reinterpret_cast<Nka *>(h);
	if (!ok_nka(k))
		return FS_ERR_BAD_HANDLE;
	reset_subspace(k);
	return FS_OK;
}

// op::nka::apply (nka.hh:64-137)
FS_API int fs_nka_apply(fs_nka h, fs_vec fh, fs_vec uh, fs_solve_info *info) {
	Nka *k = reinterpret_cast<Nka *>(h);
	Vec *f = reinterpret_cast<Vec *>(fh), *u = reinterpret_cast<Vec *>(uh);
	if (!ok_nka(k) || !ok_vec(f) || !ok_vec(u) || !info)
		return FS_ERR_BAD_HANDLE;
	Ctx *ctx = k->ctx;
	if (f->n != k->n || u->n != k->n || f->dtype != FS_F64 || u->dtype != FS_F64)
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_nka_apply: FP64 vectors of the operator's size");
	std::memset(info, 0, sizeof(*info));
	info->status = FS_STATUS_UNKNOWN;
	const fs_nka_settings &s = k->set;
	FS_TRY(neg_residual(k, f, u, k->res));
	double res_norm;
	FS_TRY(fs_vec_l2norm(hv(k->res), &res_norm));
	info->res_norm_initial = (float)res_norm;
	if (res_norm < s.base.atol) {
		info->status = FS_CONVERGED_ATOL;
		return FS_OK;
	}
	FS_TRY(fs_vec_copy(hv(u), hv(k->sol)));
	for (int iter = 0; iter < s.base.maxiter; ++iter) {
		if (k->P) {
			fs_solve_info pinfo;
			FS_TRY(fs_krylov_apply(reinterpret_cast<fs_solver>(k->P), hv(k->res), hv(k->cor), &pinfo));
		}
		else
			FS_TRY(fs_vec_copy(hv(k->res), hv(k->cor)));
		FS_TRY(compute_correction(k, k->cor));
		FS_TRY(fs_vec_axpy(-1.0, hv(k->cor), hv(k->sol), hv(k->sol)));
		FS_TRY(neg_residual(k, f, k->sol, k->res));
		FS_TRY(fs_vec_l2norm(hv(k->res), &res_norm));
		if (!std::isfinite(res_norm))
			return set_err(ctx, FS_ERR_NON_FINITE, "NKA: non-finite residual norm");
		if (res_norm < s.base.atol) {
			info->iters = iter + 1;
			info->status = FS_CONVERGED_ATOL;
			break;
		}
		if (res_norm < s.base.rtol * info->res_norm_initial) {
			info->iters = iter + 1;
			info->status = FS_CONVERGED_RTOL;
			break;
		}
		if (k->diag && k->diag(k->diag_user, hv(k->sol), res_norm)) {
			info->status = FS_CONVERGED_USER;
			info->iters = iter + 1;
			break;
		}
	}
	info->res_norm_final = (float)res_norm;
	double sn;
	FS_TRY(fs_vec_l2norm(hv(k->sol), &sn));
	info->sol_norm_final = (float)sn;
	return fs_vec_copy(hv(k->sol), hv(u));
}

FS_API int fs_nka_destroy(fs_nka h) {
	Nka *k = reinterpret_cast<Nka *>(h);
	if (!ok_nka(k))
		return FS_ERR_BAD_HANDLE;
	for (Vec *p : {k->sol, k->res, k->cor})
		if (p)
			fs_vec_destroy(hv(p));
	for (Vec *p : k->w)
		if (p)
			fs_vec_destroy(hv(p));
	for (Vec *p : k->v)
		if (p)
			fs_vec_destroy(hv(p));
	k->magic = 0;
	delete k;
	return FS_OK;
}

}  // extern "C"
