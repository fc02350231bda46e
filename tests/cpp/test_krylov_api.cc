// The C++ mirror of flecsolve's Krylov API (include/flecsolve_gb300/
// flecsolve.hh) driving the device solvers, written the way the reference's
// own tests are (flecsolve/solvers/test/cg.cc, gmres.cc, bicgstab.cc,
// flecsolve/vectors/test/flecsi_vector.cc).  Prints one PASS/FAIL line per
// check; the exit status is the number of failures.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "flecsolve_gb300/flecsolve.hh"

// seeded problem generators of libfsproblems.so
extern "C" {
int64_t fsp_grid_rows(int dim, int64_t n);
int64_t fsp_grid_nnz(int dim, int64_t n);
int64_t fsp_grid_faces(int dim, int64_t n);
void fsp_faces_const(int dim, int64_t n, double c, double *faces);
void fsp_faces_lognormal(int dim, int64_t n, double mu, double sigma, uint64_t seed, double *faces,
                         double *cells);
void fsp_assemble_diffusion(int dim, int64_t n, const double *faces, int64_t *rowptr, int32_t *col,
                            double *val);
void fsp_assemble_convdiff3d(int64_t n, double pe_max, uint64_t seed, int64_t *rowptr, int32_t *col,
                             double *val, double *vel);
void fsp_uniform(uint64_t seed, int64_t n, double lo, double hi, double *out);
}

using namespace flecsolve;

static int failures = 0;
static void expect(bool ok, const char *what) {
	std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
	if (!ok)
		++failures;
}

struct host_csr {
	std::size_t n;
	std::vector<int64_t> rp;
	std::vector<int32_t> col;
	std::vector<double> val;
};

static host_csr diffusion(int dim, int64_t n, bool lognormal) {
	host_csr A;
	A.n = fsp_grid_rows(dim, n);
	std::vector<double> faces(fsp_grid_faces(dim, n));
	if (lognormal)
		fsp_faces_lognormal(dim, n, 0.0, 1.0, 2, faces.data(), nullptr);
	else
		fsp_faces_const(dim, n, 1.0, faces.data());
	A.rp.resize(A.n + 1);
	A.col.resize(fsp_grid_nnz(dim, n));
	A.val.resize(A.col.size());
	fsp_assemble_diffusion(dim, n, faces.data(), A.rp.data(), A.col.data(), A.val.data());
	return A;
}

static host_csr convdiff(int64_t n) {
	host_csr A;
	A.n = n * n * n;
	A.rp.resize(A.n + 1);
	A.col.resize(fsp_grid_nnz(3, n));
	A.val.resize(A.col.size());
	fsp_assemble_convdiff3d(n, 5.0, 4, A.rp.data(), A.col.data(), A.val.data(), nullptr);
	return A;
}

// cg.cc:16-54: with b = 0 the error is x itself; CG must decrease its A-norm
// monotonically, and the diagnostic runs once per iteration
struct anorm_diagnostic {
	anorm_diagnostic(const mat::csr &A, const vec::device_vec &x0, const context &c)
		: A(A), Ax(c, x0.local_size()) {
		A.apply(x0, Ax);
		e_prev = std::sqrt(x0.dot(Ax).get());
	}
	bool operator()(const vec::device_vec &x, double) {
		A.apply(x, Ax);
		double e = std::sqrt(x.dot(Ax).get());
		monotonic_fail = monotonic_fail || (e > e_prev);
		e_prev = e;
		++iter;
		return false;
	}
	const mat::csr &A;
	vec::device_vec Ax;
	double e_prev = 0;
	int iter = 0;
	bool monotonic_fail = false;
};

int main() {
	context ctx;

	// ------------------------------------------- vector closed forms --
	{
		// flecsi_vector.cc:21-57, 309-401 on 32 dofs
		std::vector<double> gx(32), gy(32), gz(32);
		for (int i = 0; i < 32; ++i) {
			gx[i] = i;
			gy[i] = 2.0 * i;
			gz[i] = 3.0 * i;
		}
		vec::device_vec x(ctx, gx), y(ctx, gy), z(ctx, gz), tmp(ctx, 32);
		tmp.add(x, z);
		auto h = tmp.download();
		bool ok = true;
		for (int i = 0; i < 32; ++i)
			ok = ok && h[i] == 4.0 * i;
		expect(ok, "vec add");
		tmp.add_scalar(y, -7);
		expect(tmp.min().get() == -7, "vec min == -7");
		expect(z.max().get() == 93, "vec max == 93");
		x.set_scalar(1.5);
		y.set_scalar(3.8);
		expect(std::fabs(x.dot(y).get() - 32 * 1.5 * 3.8) < 1e-8, "vec dot");
		x.set_scalar(-3.141719);
		expect(std::fabs(x.l1norm().get() - 32 * 3.141719) < 1e-8, "vec l1norm");
		expect(std::fabs(x.l2norm().get() - std::sqrt(32.0) * 3.141719) < 1e-8, "vec l2norm");
	}

	// ------------------------------------------- vec::multi --------------
	{
		vec::multi m(ctx, {100, 7, 33});
		m.get(0).set_scalar(1.0);
		m.get(1).set_scalar(-2.0);
		m.get(2).set_scalar(0.5);
		expect(std::fabs(m.dot(m).get() - (100 + 7 * 4 + 33 * 0.25)) < 1e-12, "multi dot = sum of component dots");
		expect(std::fabs(m.l2norm().get() - std::sqrt(100 + 7 * 4 + 33 * 0.25)) < 1e-12, "multi l2norm");
		expect(m.min().get() == -2.0 && m.max().get() == 1.0, "multi min/max over components");
		auto w = m.whole().download();
		expect(w.size() == 140 && w[100] == -2.0 && w[139] == 0.5, "multi components are views of one vector");
	}

	// ------------------------------------------- CG (cg.cc style) --------
	{
		host_csr H = diffusion(2, 64, false);
		mat::csr A(ctx, H.n, H.n, H.rp, H.col, H.val);
		vec::device_vec b(ctx, H.n), x(ctx, H.n);
		b.set_scalar(0.0);
		x.set_random(7);
		anorm_diagnostic diag{A, x, ctx};
		cg::settings s{2000, 1e-9f, 1e-9f, false};  // cg.cfg
		auto slv_op = cg::solver(s, cg::make_work(b))(op::ref(A), op::I, std::ref(diag));
		auto info = slv_op(b, x);
		expect(info.status == solve_info::stop_reason::converged_rtol, "cg converged (b = 0, x0 random)");
		expect(!diag.monotonic_fail, "cg A-norm error monotone");
		expect(info.iters == diag.iter, "cg diagnostic called once per iteration");
	}
	{
		// the reference's iteration count on the 128^2 Poisson problem
		// (tests/golden: 389 with Jacobi, rtol 1e-8, zero guess)
		host_csr H = diffusion(2, 128, false);
		mat::csr A(ctx, H.n, H.n, H.rp, H.col, H.val);
		std::vector<double> hb(H.n);
		fsp_uniform(1, (int64_t)H.n, -1.0, 1.0, hb.data());
		vec::device_vec b(ctx, hb), x(ctx, H.n);
		auto info = cg::solver(cg::settings{2000, 1e-8f, 0.f, true}, cg::make_work(b))(op::ref(A), jacobi)(b, x);
		expect(info.success() && std::abs(info.iters - 389) <= 2, "cg jacobi poisson2d-128: 389 +- 2 iterations");
		vec::device_vec d = A.Dinv(ctx);
		auto info2 = cg::solver(cg::settings{2000, 1e-8f, 0.f, true}, cg::make_work(b))(op::ref(A), d)(b, x);
		expect(info2.iters == info.iters, "cg with the D^-1 vector == cg with jacobi");
		auto info3 = mixed::cg_solver(cg::settings{2000, 1e-8f, 0.f, true}, cg::make_work(b))(op::ref(A), jacobi)(b, x);
		expect(info3.success() && std::abs(info3.iters - info.iters) <= 2, "mixed cg: same iteration count");
	}

	// ------------------------------------------- BiCGSTAB ----------------
	{
		host_csr H = convdiff(16);
		mat::csr A(ctx, H.n, H.n, H.rp, H.col, H.val);
		vec::device_vec b(ctx, H.n), x(ctx, H.n);
		b.set_random(0);
		x.set_random(1);
		bicgstab::settings s{{200, 1e-9f, 0.f, false}};  // bicgstab.cfg
		bicgstab::solver slv(s, bicgstab::make_work(b));
		auto info = slv(op::ref(A))(b, x);
		expect(info.status == solve_info::stop_reason::converged_rtol, "bicgstab converged_rtol");
	}

	// ------------------------------------------- GMRES (gmres.cc style) --
	{
		host_csr H = convdiff(12);
		mat::csr A(ctx, H.n, H.n, H.rp, H.col, H.val);
		vec::device_vec b(ctx, H.n), x(ctx, H.n);
		std::vector<double> hx(H.n);
		fsp_uniform(1, (int64_t)H.n, 0.0, 1.0, hx.data());
		b.set_random(0);
		x.upload(hx);
		gmres::settings sr{{100, 1e-4f, 0.f, false}, 50, gmres::precond_side::right, true};
		gmres::solver slv(sr, gmres::make_work(b));
		auto info_restart = slv(op::ref(A))(b, x);
		x.upload(hx);
		slv.settings.maxiter = 50;
		slv(op::ref(A))(b, x);
		slv.settings.maxiter = 100;
		slv.settings.max_krylov_dim = 100;
		slv.settings.restart = false;
		auto slv1 = slv(op::ref(A));
		auto info = slv1.apply(b, x);
		expect(info_restart.success(), "gmres restarted run converged");
		expect(50 + info.iters == info_restart.iters, "gmres restart consistency: iterations");
		expect(info.res_norm_final == info_restart.res_norm_final, "gmres restart consistency: residual");
		gmres::settings bad{{10, 1e-4f, 0.f, false}, 5, gmres::precond_side::right, false};
		bool threw = false;
		try {
			gmres::solver(bad, gmres::make_work(b))(op::ref(A));
		}
		catch (const fs_error &e) {
			threw = e.status == FS_ERR_BREAKDOWN;
		}
		expect(threw, "gmres validate(): restart = false with maxiter > max_krylov_dim rejected");
	}
	{
		// NKA with a CG preconditioner, bound as solvers/test/nka.cc:72-80
		// binds it (b = 1, x0 = 3, the settings of solvers/test/nka.cfg), on
		// the 64^2 Poisson operator: the reference takes 34 iterations
		// (tests/golden/nka_golden.json)
		host_csr H = diffusion(2, 64, false);
		mat::csr A(ctx, H.n, H.n, H.rp, H.col, H.val);
		vec::device_vec b(ctx, H.n), x(ctx, H.n);
		b.set_scalar(1.);
		x.set_scalar(3.);
		cg::settings pre{11, 1e-9f, 1e-9f, true};
		nka::settings nnl{};
		nnl.maxiter = 100;
		nnl.atol = 1e-6f;
		nnl.max_dim = 5;
		nnl.angle_tol = 0.2;
		nnl.use_zero_guess = false;
		auto P = cg::solver(pre, cg::make_work(b))(op::ref(A));
		auto slv = nka::solver(nnl, nka::make_work(nka::dim_bound<5>, b))(op::ref(A), op::ref(P));
		auto info = slv(b, x);
		expect(info.status == solve_info::stop_reason::converged_atol && std::abs(info.iters - 34) <= 2,
		       "nka + cg preconditioner on poisson2d-64: 34 +- 2 iterations");
		nka::settings bad = nnl;
		bad.max_dim = 0;
		bool threw = false;
		try {
			nka::solver(bad, nka::make_work(b))(op::ref(A), op::ref(P));
		}
		catch (const fs_error &e) {
			threw = e.status == FS_ERR_BREAKDOWN;
		}
		expect(threw, "nka settings::validate: max_dim = 0 rejected");
	}
	{
		// mat::io::matrix_market as the reference's tests load an operator
		// (solvers/test/cg.cc reads SuiteSparse files the same way)
		const char *fname = std::getenv("FS_MM_FIXTURE");
		if (fname) {
			auto A = mat::io::matrix_market<>::read(fname).tocsr();
			mat::io::matrix_market<>::definition def(fname);
			std::vector<std::size_t> rng(70);
			for (std::size_t i = 0; i < rng.size(); ++i)
				rng[i] = 50 + i;
			auto part = def.matrix(rng);
			expect(A.rows() == 216 && def.num_cols() == 216 && part.rows() == 70 &&
			           part.rowptr.back() == A.rowptr[120] - A.rowptr[50],
			       "matrix_market: read(...).tocsr() and definition::matrix(range)");
			mat::csr dA(ctx, A);
			vec::device_vec b(ctx, 216), x(ctx, 216);
			b.set_scalar(1.0);
			auto info = cg::solver(cg::settings{500, 1e-10f, 0.f, true}, cg::make_work(b))(op::ref(dA),
			                                                                             jacobi)(b, x);
			expect(info.success(), "cg on a MatrixMarket operator converged");
			bool threw = false;
			try {
				mat::io::matrix_market<>::read("/nonexistent.mtx");
			}
			catch (const fs_error &e) {
				threw = e.status == FS_ERR_IO;
			}
			expect(threw, "matrix_market: a missing file raises FS_ERR_IO");
		}
	}
	{
		// physics: the finite-volume operators on fields, as
		// physics/test/fvm_diffusion.cc builds them, and the same expression
		// as the matrix-free operator of a CG solve
		using namespace physics;
		const context &pc = ctx;
		fvm_mesh m(pc, {12, 10, 8}, {{{0.0, 1.0}, {0.0, 2.0}, {0.0, 0.5}}});
		const std::size_t N = m.dofs();
		auto faces = m.face_fields(pc);
		auto a = m.cell_field(pc, 1.0);
		auto expr = op_expr(bc<dirichlet, x_axis, boundary_low>::create({0.0}, m),
		                    bc<dirichlet, x_axis, boundary_high>::create({0.0}, m),
		                    bc<neumann, y_axis, boundary_low>::create({0.0}, m),
		                    bc<neumann, y_axis, boundary_high>::create({0.0}, m),
		                    bc<neumann, z_axis, boundary_low>::create({0.0}, m),
		                    bc<neumann, z_axis, boundary_high>::create({0.0}, m),
		                    coefficient<constant_coefficient>::create({2.0}, faces, m),
		                    diffusion::create({&a, &faces, 1.0, 0.25}, m));
		std::vector<double> xs(N);
		fsp_uniform(11, (int64_t)N, -1.0, 1.0, xs.data());
		vec::device_vec x(pc, xs), y(pc, N), px(pc, N);
		auto u = m.cell_field(pc), v = m.cell_field(pc);
		m.unpack(x, u);
		expr.apply(u, v);
		m.pack(v, px);
		auto A = expr.matrix_free();
		A.apply(x, y);
		auto hy = y.download(), hv = px.download();
		bool same = true;
		for (std::size_t i = 0; i < N; ++i)
			same = same && std::memcmp(&hy[i], &hv[i], sizeof(double)) == 0;
		expect(same, "physics: the matrix-free operator equals op_expr(bc..., coefficient, diffusion) bit for bit");
		// zero-flux faces, no source: a constant field has no flux
		auto u1 = m.cell_field(pc, 3.0), v1 = m.cell_field(pc);
		auto neu = op_expr(bc<neumann, x_axis, boundary_low>::create({0.0}, m),
		                   bc<neumann, x_axis, boundary_high>::create({0.0}, m),
		                   bc<neumann, y_axis, boundary_low>::create({0.0}, m),
		                   bc<neumann, y_axis, boundary_high>::create({0.0}, m),
		                   bc<neumann, z_axis, boundary_low>::create({0.0}, m),
		                   bc<neumann, z_axis, boundary_high>::create({0.0}, m),
		                   coefficient<constant_coefficient>::create({1.0}, faces, m),
		                   diffusion::create({&a, &faces, 1.0, 0.0}, m));
		neu.apply(u1, v1);
		vec::device_vec pv(pc, N);
		m.pack(v1, pv);
		expect(pv.l2norm().get() == 0.0, "physics: zero-flux boundaries give no flux for a constant field");
		vec::device_vec b(pc, xs), sol(pc, N);
		auto info = cg::solver(cg::settings{2000, 1e-8f, 0.f, true}, cg::make_work(b))(op::ref(A), jacobi)(b, sol);
		vec::device_vec r(pc, N);
		A.residual(b, sol, r);
		expect(info.success() && r.l2norm().get() <= 1e-8 * b.l2norm().get() * 1.01,
		       "physics: jacobi cg on the matrix-free operator converged");
	}
	{
		// time_integrator::bdf as time-integrators/test/implicit.cc drives it:
		// the decay u' = -u from 3 at implicit.cfg's settings
		using namespace time_integrator;
		struct rate_op {
			double lambda, gamma = 1.0;
			void apply_rhs(const vec::device_vec &x, vec::device_vec &y) const { y.scale(lambda, x); }
			void set_scaling(double g) { gamma = g; }
		};
		struct rate_solver {
			op::handle<rate_op> F;
			solve_info apply(const vec::device_vec &b, vec::device_vec &x) const {
				const double rhs = b.min().get();
				x.set_scalar(rhs / (1. - F.get().lambda * F.get().gamma));
				solve_info i;
				i.status = solve_info::stop_reason::converged_atol;
				return i;
			}
		};
		auto run = [&](bdf::method m, int &steps, int &rejects, double &err) {
			bdf::settings s;
			s.initial_time = 0.0;
			s.final_time = 1.0;
			s.initial_dt = 0.5;
			s.max_steps = 1000;
			s.min_dt = 0.001;
			s.max_dt = 0.5;
			s.timestep_strategy = bdf::strategy::truncation_error;
			s.integrator = m;
			s.starting_integrator = bdf::method::cn;
			s.time_trunc_err_norm = bdf::norm_type::inf;
			s.predictor = bdf::predictor::leapfrog;
			s.problem_scales = {1.};
			s.time_rtol = 1e-7;
			s.time_atol = 1e-5;
			s.time_error_scaling = bdf::error_scaling::fixed_resolution;
			auto F = op::make_shared<rate_op>(rate_op{-1.0});
			auto solver = op::make_shared<rate_solver>(rate_solver{F});
			vec::device_vec x(ctx, 1), xnew(ctx, 1);
			bdf::integrator ti(bdf::parameters(s, F, bdf::make_work(x), solver));
			x.set_scalar(3.0);
			double dt = ti.get_current_dt();
			bool first = true;
			while (ti.get_current_time() < ti.get_final_time()) {
				ti.advance(dt, first, x, xnew);
				const bool good = ti.check_solution();
				if (good) {
					ti.update();
					std::swap(x, xnew);
					first = false;
				}
				dt = ti.get_next_dt(good);
			}
			steps = ti.get_current_step();
			rejects = ti.num_step_rejects();
			err = std::abs(3.0 * std::exp(-1.0) - x.max().get());
		};
		int steps = 0, rejects = 0;
		double err = 1.0;
		run(bdf::method::bdf2, steps, rejects, err);
		expect(err < 1e-3 && steps <= 49 && rejects <= 7, "bdf2: implicit.cc expectations (err < 1e-3, <= 49 steps, <= 7 rejects)");
		run(bdf::method::bdf5, steps, rejects, err);
		expect(err < 1e-7 && steps == 48 && rejects == 14, "bdf5: implicit.cc expectations (err < 1e-7, 48 steps, 14 rejects)");
		// the heat equation u' = -A u, backward Euler with the device time operator
		host_csr H = diffusion(2, 16, false);
		for (auto &v : H.val)
			v = -v;
		mat::csr J(ctx, H.n, H.n, H.rp, H.col, H.val);
		bdf::settings hs;
		hs.initial_time = 0.0;
		hs.final_time = 0.1;
		hs.initial_dt = 0.01;
		hs.max_dt = 0.01;
		hs.max_steps = 100;
		hs.timestep_strategy = bdf::strategy::constant;
		hs.integrator = hs.starting_integrator = bdf::method::be;
		hs.problem_scales = {1.};
		fs_krylov_settings ks;
		fs_krylov_settings_default(&ks);
		ks.base = {1000, 1e-12f, 0.f, 0};
		bdf::linear_integrator ht(hs, J, FS_CG, ks, true);
		vec::device_vec u(ctx, H.n), unew(ctx, H.n);
		u.set_scalar(1.0);
		double dt = ht.get_current_dt();
		bool first = true;
		while (ht.get_current_time() < ht.get_final_time()) {
			ht.advance(dt, first, u, unew);
			const bool good = ht.check_solution();
			if (good) {
				ht.update();
				std::swap(u, unew);
				first = false;
			}
			dt = ht.get_next_dt(good);
		}
		expect(std::abs(ht.get_current_time() - 0.1) < 1e-12 && u.max().get() < 1.0 && u.min().get() > 0.0,
		       "bdf linear form: backward-Euler heat reaches the final time, decaying and positive");
	}
	std::printf("%d failure(s)\n", failures);
	return failures;
}
