// ORACLE -- test infrastructure only.
//
// Runs the reference's own, unmodified serial Krylov templates
// (flecsolve/solvers/{cg,bicgstab,gmres}.hh over vec::seq_vec and
// mat::csr<double>) on a problem read from a binary file, and writes the
// solve_info, the residual history seen by the diagnostic and the solution.
// Built by oracle/Makefile against the reference headers plus the stand-in
// declarations in oracle/ref_shim/; only used to produce and check the
// golden fixtures under tests/golden/ and to pin oracle/krylov_oracle.c.
//
// Input file (little endian):
//   int64 n, int64 nnz, int64 rowptr[n+1], int32 col[nnz], double val[nnz],
//   double b[n], double x0[n]
// Command line:
//   ref_driver <in> <out> <cg|bicgstab|gmres|fcg> <maxiter> <rtol> <zero_guess>
//              <none|jacobi|cg<k>> [krylov_dim left|right restart]
// cg<k> (fcg only): the preconditioner is the reference's cg::solver with
// maxiter k, rtol 0, a zero guess and D^-1, bound as an operator (the
// nested-solver pattern of flecsolve/solvers/test/nka.cc:72-80).
// Output file:
//   int32 status, iters, restarts; float res0, res, sol0, sol, rhs;
//   int64 nhist; double hist[nhist]; double x[n]
// Timing (bench.py's reference arm): with REF_DRIVER_TIMES=<file> set, the
// diagnostic also takes a steady-clock time stamp at every call (the
// reference's loops call it once per iteration), and the driver writes
//   int64 nstamp; double seconds_since_solve_start[nstamp]; double total
// where total is the wall time of the whole solver call (set-up included).
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "flecsolve/matrices/seq.hh"
#include "flecsolve/vectors/seq.hh"
#include "flecsolve/solvers/cg.hh"
#include "flecsolve/solvers/bicgstab.hh"
#include "flecsolve/solvers/gmres.hh"

flecsi::scheduler * flecsi::scheduler::instance = nullptr;

using namespace flecsolve;

namespace {

template<class T>
void rd(std::FILE * f, T * p, std::size_t n) {
	if (std::fread(p, sizeof(T), n, f) != n)
		throw std::runtime_error("short read");
}

using clk = std::chrono::steady_clock;

struct recorder {
	std::vector<double> * hist;
	std::vector<double> * stamps; // null unless timing was asked for
	clk::time_point t0;
	template<class V>
	bool operator()(const V &, double r) const {
		if (stamps)
			stamps->push_back(std::chrono::duration<double>(clk::now() - t0).count());
		hist->push_back(r);
		return false;
	}
};

} // namespace

int main(int argc, char ** argv) {
	if (argc < 8) {
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
	// D^-1 the way flecsolve/util/test/mesh.hh:123-140 builds it
	mat::csr<double> D{N, N};
	D.resize(N);
	{
		auto [rowptr, colind, values] = A.rep();
		for (std::size_t i = 0; i < N; ++i) {
			for (std::size_t off = rowptr[i]; off < rowptr[i + 1]; ++off)
				if (colind[off] == i) {
					D.data.values()[i] = 1.0 / values[off];
					D.data.indices()[i] = i;
				}
			D.data.offsets()[i + 1] = i + 1;
		}
	}
	op::core<mat::csr<double>> Aop(std::move(A));
	op::core<mat::csr<double>> Pop(std::move(D));

	vec::seq_vec<double> b{N}, x{N};
	for (std::size_t i = 0; i < N; ++i) {
		b[i] = bh[i];
		x[i] = xh[i];
	}

	const std::string which = argv[3];
	const int maxiter = std::atoi(argv[4]);
	const float rtol = std::strtof(argv[5], nullptr);
	const bool zero_guess = std::atoi(argv[6]) != 0;
	const bool jacobi = std::string(argv[7]) == "jacobi";

	std::vector<double> hist, stamps;
	const char * times_path = std::getenv("REF_DRIVER_TIMES");
	recorder diag{&hist, times_path ? &stamps : nullptr, clk::now()};
	solve_info info;
	int assert_failed = 0;
	diag.t0 = clk::now();
	try {
		if (which == "cg") {
			cg::settings s{maxiter, rtol, 0.f, zero_guess};
			vec::seq_work<double, cg::nwork> w{b};
			if (jacobi)
				info = cg::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = cg::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else if (which == "bicgstab") {
			bicgstab::settings s{{maxiter, rtol, 0.f, zero_guess}};
			vec::seq_work<double, bicgstab::nwork> w{b};
			if (jacobi)
				info = bicgstab::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = bicgstab::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else if (which == "fcg") {
			fcg::settings s{maxiter, rtol, 0.f, zero_guess};
			vec::seq_work<double, fcg::nwork> w{b};
			const std::string pname = argv[7];
			if (pname.rfind("cg", 0) == 0) {
				cg::settings ps{std::atoi(pname.c_str() + 2), 0.f, 0.f, true};
				auto inner = cg::solver(ps, vec::seq_work<double, cg::nwork>{b})(op::ref(Aop),
				                                                               op::ref(Pop));
				info = fcg::solver(s, std::move(w))(op::ref(Aop), op::ref(inner), diag)(b, x);
			}
			else if (jacobi)
				info = fcg::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = fcg::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else if (which == "gmres") {
			if (argc < 11)
				return 2;
			gmres::settings s{{maxiter, rtol, 0.f, zero_guess},
			                  std::atoi(argv[8]),
			                  std::string(argv[9]) == "left" ? gmres::precond_side::left
			                                                  : gmres::precond_side::right,
			                  std::atoi(argv[10]) != 0};
			std::array<vec::seq_vec<double>, gmres::nwork> w;
			for (auto & v : w)
				v.data.resize(N);
			if (jacobi)
				info = gmres::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = gmres::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else
			return 2;
	}
	catch (const std::runtime_error & e) {
		std::fprintf(stderr, "assert: %s\n", e.what());
		assert_failed = 1;
	}
	const double total = std::chrono::duration<double>(clk::now() - diag.t0).count();
	if (times_path) {
		std::FILE * t = std::fopen(times_path, "wb");
		if (!t)
			return 5;
		int64_t ns = static_cast<int64_t>(stamps.size());
		std::fwrite(&ns, sizeof(int64_t), 1, t);
		std::fwrite(stamps.data(), sizeof(double), stamps.size(), t);
		std::fwrite(&total, sizeof(double), 1, t);
		std::fclose(t);
	}

	std::FILE * o = std::fopen(argv[2], "wb");
	if (!o)
		return 4;
	int32_t head[3] = {assert_failed ? 100 : static_cast<int32_t>(info.status),
	                   info.iters, info.restarts};
	float norms[5] = {info.res_norm_initial, info.res_norm_final,
	                  info.sol_norm_initial, info.sol_norm_final, info.rhs_norm};
	int64_t nh = static_cast<int64_t>(hist.size());
	std::fwrite(head, sizeof(int32_t), 3, o);
	std::fwrite(norms, sizeof(float), 5, o);
	std::fwrite(&nh, sizeof(int64_t), 1, o);
	std::fwrite(hist.data(), sizeof(double), hist.size(), o);
	for (std::size_t i = 0; i < N; ++i) {
		double v = x[i];
		std::fwrite(&v, sizeof(double), 1, o);
	}
	std::fclose(o);
	return 0;
}
