// ORACLE -- test infrastructure only.
//
// Runs the reference's own, unmodified NKA (flecsolve/solvers/nka.hh) over
// vec::seq_vec and mat::csr<double>, preconditioned by the reference's CG
// solver (flecsolve/solvers/cg.hh), as solvers/test/nka.cc:72-80 sets it up:
// P = cg::solver(pc_settings, work)(A) applied as the preconditioner of
// nka::solver(settings, work)(A, op::ref(P)).  Writes the solve_info, the
// residual history seen by the diagnostic and the solution.  Built by
// oracle/Makefile against the reference headers plus the stand-ins in
// oracle/ref_shim/; only used to produce the golden fixtures under
// tests/golden/.
//
// Input file: as ref_driver (int64 n, nnz; int64 rowptr[n+1]; int32 col[nnz];
// double val[nnz], b[n], x0[n]).
// Command line:
//   ref_nka <in> <out> <maxiter> <atol> <max_dim> <angle_tol> <pc_maxiter> <pc_rtol>
//           [use_damping adaptive_damping damping_factor]
// Output file: int32 status, iters; float res0, res, sol; int64 nhist;
// double hist[nhist]; double x[n]
#include <array>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "flecsolve/matrices/seq.hh"
#include "flecsolve/vectors/seq.hh"
#include "flecsolve/solvers/cg.hh"
#include "flecsolve/solvers/nka.hh"

flecsi::scheduler * flecsi::scheduler::instance = nullptr;

using namespace flecsolve;

namespace {

template<class T>
void rd(std::FILE * f, T * p, std::size_t n) {
	if (std::fread(p, sizeof(T), n, f) != n)
		throw std::runtime_error("short read");
}

struct recorder {
	std::vector<double> * hist;
	template<class V>
	bool operator()(const V &, double r) const {
		hist->push_back(r);
		return false;
	}
};

constexpr int kDim = 10;  // dimension bound of the work (solvers/test/nka.cc:74 uses 5 and 10)

} // namespace

int main(int argc, char ** argv) {
	if (argc != 9 && argc != 12) {
		std::fprintf(stderr, "usage: see header\n");
		return 2;
	}
	std::FILE * f = std::fopen(argv[1], "rb");
	if (!f)
		return 3;
	int64_t n, nnz;
	rd(f, &n, 1);
	rd(f, &nnz, 1);
	std::vector<int64_t> rp(n + 1);
	std::vector<int32_t> ci(nnz);
	std::vector<double> va(nnz), bh(n), xh(n);
	rd(f, rp.data(), n + 1);
	rd(f, ci.data(), nnz);
	rd(f, va.data(), nnz);
	rd(f, bh.data(), n);
	rd(f, xh.data(), n);
	std::fclose(f);

	const std::size_t N = n;
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
	vec::seq_vec<double> b{N}, x{N};
	for (std::size_t i = 0; i < N; ++i) {
		b[i] = bh[i];
		x[i] = xh[i];
	}

	nka::settings s{};
	s.maxiter = std::atoi(argv[3]);
	s.rtol = 0.f;
	s.atol = std::strtof(argv[4], nullptr);
	s.use_zero_guess = false;
	s.max_dim = std::atoi(argv[5]);
	s.angle_tol = std::strtod(argv[6], nullptr);
	s.max_fun_evals = 0;
	s.freeze_pc = true;
	s.use_qr = false;
	s.use_damping = argc == 12 && std::atoi(argv[9]) != 0;
	s.adaptive_damping = argc == 12 && std::atoi(argv[10]) != 0;
	s.damping_factor = argc == 12 ? std::strtod(argv[11], nullptr) : 1.;
	const float pc_rtol = std::strtof(argv[8], nullptr);
	cg::settings ps{std::atoi(argv[7]), pc_rtol, pc_rtol, true};

	std::vector<double> hist;
	recorder diag{&hist};
	solve_info info;
	{
		vec::seq_work<double, cg::nwork> pw{b};
		auto P = cg::solver(ps, std::move(pw))(op::ref(Aop));
		std::array<vec::seq_vec<double>, nka::nwork + 2 * (kDim + 1)> w;
		for (auto & v : w)
			v = vec::seq_vec<double>{N};
		auto slv = nka::solver(s, std::move(w))(op::ref(Aop), op::ref(P), diag);
		info = slv(b, x);
	}

	std::FILE * o = std::fopen(argv[2], "wb");
	if (!o)
		return 4;
	int32_t st = (int32_t)info.status, it = (int32_t)info.iters;
	float r0 = info.res_norm_initial, r1 = info.res_norm_final, s1 = info.sol_norm_final;
	int64_t nh = (int64_t)hist.size();
	std::fwrite(&st, 4, 1, o);
	std::fwrite(&it, 4, 1, o);
	std::fwrite(&r0, 4, 1, o);
	std::fwrite(&r1, 4, 1, o);
	std::fwrite(&s1, 4, 1, o);
	std::fwrite(&nh, 8, 1, o);
	std::fwrite(hist.data(), 8, hist.size(), o);
	std::vector<double> xo(N);
	for (std::size_t i = 0; i < N; ++i)
		xo[i] = x[i];
	std::fwrite(xo.data(), 8, N, o);
	std::fclose(o);
	return 0;
}
