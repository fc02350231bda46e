// ORACLE -- test infrastructure only.
//
// Runs the reference's own, unmodified BDF time integrator
// (flecsolve/time-integrators/bdf.hh, bdf.cc, bdf_parameters.cc) over
// vec::seq_vec, driven the way the reference's test drives it
// (time-integrators/test/implicit.cc:90-113: advance, check_solution,
// update on a good step, get_next_dt), on one of two problems:
//  * rate: the scalar decay u' = lambda u of implicit.cc:14-73, with its
//    exact solver of the time operator;
//  * heat: u' = -A u for a CSR matrix A, the time operator
//    u - gamma f(u) = (I + gamma A) u solved by the reference's CG (no
//    preconditioner) through time_integrator::operator_adapter
//    (operator_adapter.hh:25-52).
// Writes, per attempted step, the time, dt, whether it was accepted and the
// solver's iteration count, then the final solution.  Built by
// oracle/Makefile against the reference headers and sources; only used to
// produce the golden fixtures under tests/golden/.
//
// Input file (little endian):
//   int32 problem (0 rate, 1 heat), method, starting method, predictor,
//         strategy, controller, error scaling, norm (0 inf, 1 l2, 2 l1),
//         use_pi_controller, control_timestep_variation
//   double initial_time, final_time, initial_dt, max_dt, min_dt,
//          trunc_rtol, trunc_atol, problem_scale, dt_cut_lower_bound,
//          target_relative_change
//   int32 max_steps
//   rate:  double lambda, ic, int64 n (vector length)
//   heat:  int64 n, nnz; int64 rowptr[n+1]; int32 col[nnz];
//          double val[nnz], u0[n]; int32 cg_maxiter; double cg_rtol
// Output file: int32 steps, rejects, nrecords, aborted; per record double t,
//   dt, int32 accepted, iters; then double u[n].
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

#include "flecsolve/matrices/seq.hh"
#include "flecsolve/operators/core.hh"
#include "flecsolve/solvers/cg.hh"
#include "flecsolve/time-integrators/bdf.hh"
#include "flecsolve/time-integrators/operator_adapter.hh"
#include "flecsolve/vectors/seq.hh"

flecsi::scheduler * flecsi::scheduler::instance = nullptr;

using namespace flecsolve;
using namespace flecsolve::time_integrator;

namespace {

// The reference's serial vector operations plus the one-component `apply`
// that its FleCSI operations define (vectors/operations/topo_view.hh:287-290)
// and that vec::apply (vectors/util.hh:24-36), used by the integrator's
// truncation-error norms, calls; seq_ops lacks it.
template<class Data>
struct seq_ops_apply : vec::seq_ops<Data> {
	template<class F, class... Vecs>
	static constexpr decltype(auto) apply(F && f, Vecs &&... vecs) {
		return std::forward<F>(f)(std::forward<Vecs>(vecs)...);
	}
};
struct bvec : vec::core<vec::seq_data_vec, seq_ops_apply, vec::seq_config<double, anon_var::anonymous>> {
	using base = vec::core<vec::seq_data_vec, seq_ops_apply, vec::seq_config<double, anon_var::anonymous>>;
	bvec() : base{vec::vec_t<double>{}} {}
	explicit bvec(std::size_t n) : base{vec::vec_t<double>(n)} {}
};

template<class T>
void rd(std::FILE * f, T * p, std::size_t n) {
	if (std::fread(p, sizeof(T), n, f) != n)
		throw std::runtime_error("short read");
}

// implicit.cc:14-56 (the rate operator and its exact solver)
struct rate_params {
	double lambda;
	double gamma;
};
struct rate : op::base<rate_params> {
	rate(double lambda) : op::base<rate_params>(rate_params{lambda, 1.}) {}
	template<class D, class R>
	void residual(const D & b, const R & x, R & r) const {
		apply(x, r);
		r.subtract(b, r);
	}
	template<class D, class R>
	void apply(const D & x, R & y) const {
		apply_rhs(x, y);
		y.axpy(-params.gamma, y, x);
	}
	template<class D, class R>
	void apply_rhs(const D & x, R & y) const {
		y.scale(params.lambda, x);
	}
	template<class V>
	bool is_valid(const V &) {
		return true;
	}
	double get_scaling() const { return params.gamma; }
	void set_scaling(double s) { params.gamma = s; }
	double get_rate() const { return params.lambda; }
};
struct rate_solver : op::base<> {
	rate_solver(op::handle<op::core<rate>> oph) : F(oph) {}
	template<class D, class R>
	solve_info apply(const D & b, R & x) const {
		auto rhs = b.min().get();
		const auto & o = F.get();
		auto sol = rhs / (1. - o.get_rate() * o.get_scaling());
		x.set_scalar(sol);
		solve_info info;
		info.status = solve_info::stop_reason::converged_atol;
		return info;
	}
	op::handle<op::core<rate>> F;
};

// f(u) = -A u
struct neg_matrix : op::base<> {
	explicit neg_matrix(const mat::csr<double> * A) : A(A) {}
	template<class D, class R>
	void apply(const D & x, R & y) const {
		A->apply(x, y);
		y.scale(-1.0);
	}
	const mat::csr<double> * A;
};
using heat_op = op::core<operator_adapter<neg_matrix>>;

// the reference's CG on the time operator, as a solver the integrator calls
template<class S>
struct cg_time_solver : op::base<> {
	cg_time_solver(S * slv, int * iters) : slv(slv), iters(iters) {}
	template<class D, class R>
	solve_info apply(const D & b, R & x) const {
		auto info = slv->apply(b, x);
		*iters = info.iters;
		return info;
	}
	S * slv;
	int * iters;
};

// The integrator leaves current_steprejects and prev_successive_rejects
// uninitialised (bdf.hh:56-63 sets neither) and reads them in check_solution
// and get_next_dt; it is constructed here in zero-filled storage so that they
// start at 0 / false, which is what the reference's test expectations
// (implicit.cc:126-131) correspond to.
template<class P>
auto * place(P && p) {
	using I = decltype(bdf::integrator(std::forward<P>(p)));
	static std::vector<unsigned char> store;
	store.assign(sizeof(I) + alignof(I), 0);
	void * at = store.data();
	std::size_t space = store.size();
	at = std::align(alignof(I), sizeof(I), at, space);
	return new (at) I(std::forward<P>(p));
}

struct record {
	double t, dt;
	int32_t accepted, iters;
};

// the test's loop; returns false when the integrator asserted (advance
// compares the two vectors by value, bdf.hh:76-77, so a step that leaves the
// solution unchanged aborts the run)
template<class TI, class V>
bool run(TI & ti, V & x, V & xnew, int * iters, std::vector<record> & rec) {
	auto dt = ti.get_current_dt();
	bool first_step = true;
	int guard = 0;
	while (ti.get_current_time() < ti.get_final_time() && guard++ < 100000) {
		const double t = ti.get_current_time();
		*iters = 0;
		try {
			ti.advance(dt, first_step, x, xnew);
		}
		catch (const std::runtime_error &) {
			return false;
		}
		auto good = ti.check_solution();
		rec.push_back({t, dt, good ? 1 : 0, *iters});
		if (good) {
			ti.update();
			std::swap(x, xnew);
			first_step = false;
		}
		dt = ti.get_next_dt(good);
	}
	return true;
}

} // namespace

int main(int argc, char ** argv) {
	if (argc != 3) {
		std::fprintf(stderr, "usage: ref_bdf <in> <out>\n");
		return 2;
	}
	std::FILE * f = std::fopen(argv[1], "rb");
	if (!f)
		return 2;
	int32_t e[10];
	double d[10];
	int32_t max_steps;
	rd(f, e, 10);
	rd(f, d, 10);
	rd(f, &max_steps, 1);

	bdf::settings s{};
	s.initial_time = d[0];
	s.final_time = d[1];
	s.initial_dt = d[2];
	s.max_dt = d[3];
	s.min_dt = d[4];
	s.max_steps = max_steps;
	s.integrator = static_cast<bdf::method>(e[1]);
	s.starting_integrator = static_cast<bdf::method>(e[2]);
	s.predictor = static_cast<bdf::predictor>(e[3]);
	s.timestep_strategy = static_cast<bdf::strategy>(e[4]);
	s.pi_controller_type = static_cast<bdf::controller>(e[5]);
	s.time_error_scaling = static_cast<bdf::error_scaling>(e[6]);
	s.time_trunc_err_norm = static_cast<vec::norm_type>(e[7]);
	s.use_pi_controller = e[8] != 0;
	s.control_timestep_variation = e[9] != 0;
	// implicit.cfg's remaining keys and the option defaults
	// (bdf_parameters.hh:126-155)
	s.use_predictor = true;
	s.use_initial_predictor = true;
	s.has_source_term = false;
	s.combine_timestep_estimators = false;
	s.calculate_time_trunc_error = false;
	s.dt_cut_lower_bound = d[8];
	s.dt_growth_upper_bound = 1.702;
	s.number_of_time_intervals = 100;
	s.target_relative_change = d[9];
	s.time_rtol = d[5];
	s.time_atol = d[6];
	s.problem_scales = {d[7]};

	std::vector<record> rec;
	int iters = 0;
	int steps = 0, rejects = 0;
	bool completed = true;
	std::vector<double> out;
	if (e[0] == 0) {
		double lambda, ic;
		int64_t n;
		rd(f, &lambda, 1);
		rd(f, &ic, 1);
		rd(f, &n, 1);
		std::fclose(f);
		auto F = op::make_shared<rate>(lambda);
		bvec x{(std::size_t)n}, xnew{(std::size_t)n};
		auto solver = op::make_shared<rate_solver>(F);
		std::array<bvec, bdf::work_size> work;
		for (auto & w : work)
			w.data.resize((std::size_t)n);
		auto &ti = *place(bdf::parameters(s, F, std::move(work), solver));
		x.set_scalar(ic);
		completed = run(ti, x, xnew, &iters, rec);
		steps = ti.get_current_step();
		rejects = ti.num_step_rejects();
		for (std::size_t i = 0; i < (std::size_t)n; ++i)
			out.push_back(x[i]);
	}
	else {
		int64_t n, nnz;
		rd(f, &n, 1);
		rd(f, &nnz, 1);
		std::vector<int64_t> rp(n + 1);
		std::vector<int32_t> ci(nnz);
		std::vector<double> va(nnz), u0(n);
		int32_t cg_maxiter;
		double cg_rtol;
		rd(f, rp.data(), n + 1);
		rd(f, ci.data(), nnz);
		rd(f, va.data(), nnz);
		rd(f, u0.data(), n);
		rd(f, &cg_maxiter, 1);
		rd(f, &cg_rtol, 1);
		std::fclose(f);
		const std::size_t N = (std::size_t)n;
		mat::csr<double> A{N, N};
		A.resize(nnz);
		{
			auto [rowptr, colind, values] = A.rep();
			for (std::size_t i = 0; i <= N; ++i)
				rowptr[i] = rp[i];
			for (int64_t k = 0; k < nnz; ++k) {
				colind[k] = ci[k];
				values[k] = va[k];
			}
		}
		op::core<mat::csr<double>> Aop(std::move(A));
		auto T = op::make_shared<heat_op>(&Aop);
		bvec x{N}, xnew{N};
		cg::settings cs{cg_maxiter, (float)cg_rtol, 0.f, false};
		std::array<bvec, cg::nwork> cw;
		for (auto & w : cw)
			w.data.resize(N);
		auto cgs = cg::solver(cs, std::move(cw))(op::ref(T.get()));
		auto solver = op::make_shared<cg_time_solver<decltype(cgs)>>(&cgs, &iters);
		std::array<bvec, bdf::work_size> work;
		for (auto & w : work)
			w.data.resize(N);
		auto &ti = *place(bdf::parameters(s, T, std::move(work), solver));
		for (std::size_t i = 0; i < N; ++i)
			x[i] = u0[i];
		completed = run(ti, x, xnew, &iters, rec);
		steps = ti.get_current_step();
		rejects = ti.num_step_rejects();
		for (std::size_t i = 0; i < N; ++i)
			out.push_back(x[i]);
	}
	std::FILE * o = std::fopen(argv[2], "wb");
	if (!o)
		return 2;
	int32_t head[4] = {steps, rejects, (int32_t)rec.size(), completed ? 0 : 1};
	std::fwrite(head, sizeof(int32_t), 4, o);
	for (auto & r : rec) {
		std::fwrite(&r.t, sizeof(double), 1, o);
		std::fwrite(&r.dt, sizeof(double), 1, o);
		std::fwrite(&r.accepted, sizeof(int32_t), 1, o);
		std::fwrite(&r.iters, sizeof(int32_t), 1, o);
	}
	std::fwrite(out.data(), sizeof(double), out.size(), o);
	std::fclose(o);
	return 0;
}
