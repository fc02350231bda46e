// ORACLE -- test infrastructure only.
//
// Runs the reference's own, unmodified finite-volume physics operators
// (flecsolve/physics/): the boundary operators bc<dirichlet> / bc<neumann>
// (boundary/dirichlet.hh:49-63, boundary/neumann.hh:49-74), the face
// coefficient setters (volume_diffusion/coefficient.hh:84-177) and the
// diffusion operator's three tasks update_flux / sum_cell_flux / operate
// (volume_diffusion/diffusion.hh:109-193), in the order an operator
// expression op_expr(boundaries..., coefficient, diffusion) applies them
// (expressions/operator_expression.hh:68-71), with the mesh spacing set by
// the specialization's own set_geom (specializations/fvm_narray.hh:279-289).
// The FleCSI mesh layout they run on is the stand-in in
// oracle/ref_shim/flecsi/topo/narray/interface.hh.  Built by oracle/Makefile
// against the reference headers; only used to produce the golden fixtures
// under tests/golden/.
//
// Input file (little endian):
//   int64 nx, ny, nz; double box[3][2] (x, y, z: low, high)
//   double beta, alpha
//   int32 bc_kind[6] (0 none, 1 dirichlet, 2 neumann; x low, x high, y low,
//         y high, z low, z high); double bc_value[6]
//   int32 coef_kind (0 the faces as given, 1 constant, 2 average);
//   double coef_value
//   double u[C], a[C], v[C]  (C = (nz+2)(ny+2)(nx+2), [k][j][i], i fastest)
//   double bx[F], by[F], bz[F]  (F = (nz+1)(ny+1)(nx+1))
// Output file: double u[C] (after the boundary operators), bx[F], by[F],
// bz[F] (after the coefficient setter), v[C].
//
// With `cg <maxiter> <rtol> <zero_guess>` after the file names the input also
// holds double b[N], x0[N] (N = nx ny nz, the logical cells, i fastest) and
// the program instead solves A x = b with the reference's CG
// (flecsolve/solvers/cg.hh, no preconditioner) over vec::seq_vec, A being the
// operator expression above applied to the logical cells of u, as the
// equilibrium-diffusion example solves it (examples/equilibrium_diffusion/
// include/equilibrium_diffusion.hh:319-345).  Output as ref_driver: int32
// status, iters, restarts; float res0, res, sol0, sol, rhs; int64 nhist;
// double hist[nhist]; double x[N].
#include <cstdint>
#include <cstdio>
#include <optional>
#include <stdexcept>
#include <vector>

#include "flecsolve/physics/boundary/dirichlet.hh"
#include "flecsolve/physics/boundary/neumann.hh"
#include "flecsolve/physics/volume_diffusion/coefficient.hh"
#include "flecsolve/physics/volume_diffusion/diffusion.hh"
#include "flecsolve/solvers/cg.hh"
#include "flecsolve/vectors/seq.hh"

flecsi::scheduler * flecsi::scheduler::instance = nullptr;

using namespace flecsolve::physics;
using msh = fvm_narray;

namespace {

// the vector type the operator templates are instantiated for: a cell field
// of doubles on the mesh above
struct fvm_vec {
	using scalar = double;
	struct data_t {
		using topo_t = msh;
		template<flecsi::privilege>
		using acc = flecsi::topo::field_view;
		template<flecsi::privilege>
		using acc_all = flecsi::topo::field_view;
	};
};
constexpr auto kVar = flecsolve::anon_var::anonymous;

template<class T>
void rd(std::FILE * f, T * p, std::size_t n) {
	if (std::fread(p, sizeof(T), n, f) != n)
		throw std::runtime_error("short read");
}

template<class Spec, auto Axis, auto Boundary, class... A>
void run_bc(A &&... a) {
	tasks::operator_task<bc<Spec, Axis, Boundary>>::operate(a...);
}

template<auto Axis, auto Boundary>
void boundary(int kind, msh::accessor<flecsi::ro> m, flecsi::topo::field_view u, double value) {
	if (kind == 1)
		run_bc<dirichlet<fvm_vec, kVar>, Axis, Boundary>(m, u, value);
	else if (kind == 2)
		run_bc<neumann<fvm_vec, kVar>, Axis, Boundary>(m, u, value);
}

// the operator expression op_expr(boundaries..., coefficient, diffusion) on
// the fields of one mesh
struct model {
	msh::accessor<flecsi::ro> m;
	double beta, alpha, bc_value[6], coef_value;
	std::int32_t bc_kind[6], coef_kind;
	std::size_t C, F;
	std::vector<double> u, a, v, b[3], flux[3], du;

	void apply() {
		using fv = flecsi::topo::field_view;
		const fv U{u.data()}, A{a.data()}, V{v.data()}, B[3] = {{b[0].data()}, {b[1].data()}, {b[2].data()}};
		using D = msh::domain;
		boundary<msh::x_axis, D::boundary_low>(bc_kind[0], m, U, bc_value[0]);
		boundary<msh::x_axis, D::boundary_high>(bc_kind[1], m, U, bc_value[1]);
		boundary<msh::y_axis, D::boundary_low>(bc_kind[2], m, U, bc_value[2]);
		boundary<msh::y_axis, D::boundary_high>(bc_kind[3], m, U, bc_value[3]);
		boundary<msh::z_axis, D::boundary_low>(bc_kind[4], m, U, bc_value[4]);
		boundary<msh::z_axis, D::boundary_high>(bc_kind[5], m, U, bc_value[5]);
		if (coef_kind == 1)
			tasks::operator_task<coefficient<constant_coefficient<fvm_vec, kVar>, fvm_vec>>::coef(
				m, B[0], B[1], B[2], coef_value);
		else if (coef_kind == 2)
			tasks::operator_task<coefficient<average_coefficient<fvm_vec, kVar>, fvm_vec>>::coef(
				m, U, B[0], B[1], B[2]);
		fv FX[3] = {{flux[0].data()}, {flux[1].data()}, {flux[2].data()}}, DU{du.data()};
		using T = tasks::operator_task<diffusion<fvm_vec, kVar>>;
		T::update_flux(m, U, B[0], B[1], B[2], FX[0], FX[1], FX[2]);
		T::sum_cell_flux(m, FX[0], FX[1], FX[2], DU);
		T::operate(m, beta, alpha, A, U, DU, V);
	}

	// index of logical cell r in a cell field
	std::size_t cell(std::size_t r) const {
		const std::size_t nx = m.n[0], ny = m.n[1];
		const std::size_t i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
		return ((k + 1) * (ny + 2) + (j + 1)) * (nx + 2) + (i + 1);
	}
};

// the expression as an operator on vectors of logical cells
struct physics_op : flecsolve::op::base<> {
	explicit physics_op(model * md) : md(md) {}
	template<class D, class R>
	void apply(const D & x, R & y) const {
		const std::size_t N = md->m.n[0] * md->m.n[1] * md->m.n[2];
		for (std::size_t r = 0; r < N; ++r)
			md->u[md->cell(r)] = x[r];
		md->apply();
		for (std::size_t r = 0; r < N; ++r)
			y[r] = md->v[md->cell(r)];
	}
	model * md;
};

struct recorder {
	std::vector<double> * hist;
	template<class V>
	bool operator()(const V &, double r) const {
		hist->push_back(r);
		return false;
	}
};

} // namespace

int main(int argc, char ** argv) {
	if (argc != 3 && argc != 7) {
		std::fprintf(stderr, "usage: ref_fvm <in> <out> [cg <maxiter> <rtol> <zero_guess>]\n");
		return 2;
	}
	std::FILE * f = std::fopen(argv[1], "rb");
	if (!f)
		return 2;
	model md;
	std::int64_t n[3];
	double box[3][2];
	rd(f, n, 3);
	rd(f, &box[0][0], 6);
	rd(f, &md.beta, 1);
	rd(f, &md.alpha, 1);
	rd(f, md.bc_kind, 6);
	rd(f, md.bc_value, 6);
	rd(f, &md.coef_kind, 1);
	rd(f, &md.coef_value, 1);
	md.C = (std::size_t)((n[2] + 2) * (n[1] + 2) * (n[0] + 2));
	md.F = (std::size_t)((n[2] + 1) * (n[1] + 1) * (n[0] + 1));
	md.u.resize(md.C);
	md.a.resize(md.C);
	md.v.resize(md.C);
	md.du.assign(md.C, 0.0);
	for (int k = 0; k < 3; ++k) {
		md.b[k].resize(md.F);
		md.flux[k].assign(md.F, 0.0);
	}
	rd(f, md.u.data(), md.C);
	rd(f, md.a.data(), md.C);
	rd(f, md.v.data(), md.C);
	for (auto & bb : md.b)
		rd(f, bb.data(), md.F);
	const std::size_t N = (std::size_t)(n[0] * n[1] * n[2]);
	std::vector<double> bh, xh;
	if (argc == 7) {
		bh.resize(N);
		xh.resize(N);
		rd(f, bh.data(), N);
		rd(f, xh.data(), N);
	}
	std::fclose(f);

	md.m.n = {{(std::size_t)n[0], (std::size_t)n[1], (std::size_t)n[2]}};
	msh::gbox g;
	for (int d = 0; d < 3; ++d)
		g[d] = {{box[d][0], box[d][1]}};
	md.m.set_geom(g);

	std::FILE * o = std::fopen(argv[2], "wb");
	if (!o)
		return 2;
	if (argc == 3) {
		md.apply();
		std::fwrite(md.u.data(), sizeof(double), md.C, o);
		for (auto & bb : md.b)
			std::fwrite(bb.data(), sizeof(double), md.F, o);
		std::fwrite(md.v.data(), sizeof(double), md.C, o);
		std::fclose(o);
		return 0;
	}
	using namespace flecsolve;
	op::core<physics_op> Aop(&md);
	vec::seq_vec<double> b{N}, x{N};
	for (std::size_t i = 0; i < N; ++i) {
		b[i] = bh[i];
		x[i] = xh[i];
	}
	std::vector<double> hist;
	recorder diag{&hist};
	cg::settings s{std::atoi(argv[4]), std::strtof(argv[5], nullptr), 0.f, std::atoi(argv[6]) != 0};
	vec::seq_work<double, cg::nwork> w{b};
	solve_info info = cg::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
	std::int32_t head[3] = {static_cast<std::int32_t>(info.status), info.iters, info.restarts};
	float norms[5] = {info.res_norm_initial, info.res_norm_final, info.sol_norm_initial, info.sol_norm_final,
	                  info.rhs_norm};
	std::int64_t nh = static_cast<std::int64_t>(hist.size());
	std::fwrite(head, sizeof(std::int32_t), 3, o);
	std::fwrite(norms, sizeof(float), 5, o);
	std::fwrite(&nh, sizeof(std::int64_t), 1, o);
	std::fwrite(hist.data(), sizeof(double), hist.size(), o);
	for (std::size_t i = 0; i < N; ++i) {
		double val = x[i];
		std::fwrite(&val, sizeof(double), 1, o);
	}
	std::fclose(o);
	return 0;
}
