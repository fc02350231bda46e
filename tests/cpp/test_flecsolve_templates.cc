// flecsolve's own, unmodified solver templates on device vectors.
//
// Built (where a flecsolve checkout is available: the staged copy, with the
// FleCSI/Boost stand-ins of oracle/ref_shim) against
// include/flecsolve_gb300/flecsolve_device.hh: the reference's cg.hh (CG and
// the flexible CG), bicgstab.hh and gmres.hh run over vec::device_vec and
// mat::device_csr, so every vector operation, reduction and SpMV is a
// libfsgpu.so call on the GPU.  Nothing of the reference is changed: this is
// the binding a flecsolve maintainer would add.
//
// Same command line and file formats as oracle/ref_driver (which runs the
// same templates over vec::seq_vec), so the tests compare the two runs
// directly:
//   test_flecsolve_templates <in> <out> <cg|fcg|bicgstab|gmres> <maxiter> <rtol>
//        <zero_guess> <none|jacobi|cg<k>> [krylov_dim left|right restart]
#include <array>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "flecsolve/solvers/bicgstab.hh"
#include "flecsolve/solvers/cg.hh"
#include "flecsolve/solvers/gmres.hh"
#include "flecsolve_gb300/flecsolve_device.hh"

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

void ok(int st) {
	if (st != FS_OK)
		throw std::runtime_error(fs_status_string(st));
}

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

	fs_ctx ctx = nullptr;
	ok(fs_ctx_create(0, &ctx));
	fs_csr Ah = nullptr, Dh = nullptr;
	ok(fs_csr_create(ctx, n, n, nnz, rp.data(), ci.data(), 4, va.data(), &Ah));
	// D^-1 as a one-entry-per-row CSR, as flecsolve/util/test/mesh.hh:123-140
	// builds it
	{
		std::vector<int64_t> drp(n + 1);
		std::vector<int32_t> dci(n);
		std::vector<double> dva(n, 0.0);
		for (int64_t i = 0; i < n; ++i) {
			drp[i + 1] = i + 1;
			dci[i] = static_cast<int32_t>(i);
			for (int64_t k = rp[i]; k < rp[i + 1]; ++k)
				if (ci[k] == i)
					dva[i] = 1.0 / va[k];
		}
		ok(fs_csr_create(ctx, n, n, n, drp.data(), dci.data(), 4, dva.data(), &Dh));
	}
	op::core<mat::device_csr> Aop(Ah);
	op::core<mat::device_csr> Pop(Dh);

	vec::device_vec<double> b(ctx, n), x(ctx, n);
	b.upload(bh);
	x.upload(xh);

	const std::string which = argv[3];
	const int maxiter = std::atoi(argv[4]);
	const float rtol = std::strtof(argv[5], nullptr);
	const bool zero_guess = std::atoi(argv[6]) != 0;
	const std::string pname = argv[7];
	const bool jacobi = pname == "jacobi";

	std::vector<double> hist;
	recorder diag{&hist};
	solve_info info;
	int assert_failed = 0;
	try {
		if (which == "cg") {
			cg::settings s{maxiter, rtol, 0.f, zero_guess};
			auto w = vec::make_device_work<cg::nwork>(b);
			if (jacobi)
				info = cg::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = cg::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else if (which == "fcg") {
			fcg::settings s{maxiter, rtol, 0.f, zero_guess};
			auto w = vec::make_device_work<fcg::nwork>(b);
			if (pname.rfind("cg", 0) == 0) {
				cg::settings ps{std::atoi(pname.c_str() + 2), 0.f, 0.f, true};
				auto inner = cg::solver(ps, vec::make_device_work<cg::nwork>(b))(op::ref(Aop),
				                                                                op::ref(Pop));
				info = fcg::solver(s, std::move(w))(op::ref(Aop), op::ref(inner), diag)(b, x);
			}
			else if (jacobi)
				info = fcg::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = fcg::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else if (which == "bicgstab") {
			bicgstab::settings s{{maxiter, rtol, 0.f, zero_guess}};
			auto w = vec::make_device_work<bicgstab::nwork>(b);
			if (jacobi)
				info = bicgstab::solver(s, std::move(w))(op::ref(Aop), op::ref(Pop), diag)(b, x);
			else
				info = bicgstab::solver(s, std::move(w))(op::ref(Aop), op::I, diag)(b, x);
		}
		else if (which == "gmres") {
			if (argc < 11)
				return 2;
			gmres::settings s{{maxiter, rtol, 0.f, zero_guess},
			                  std::atoi(argv[8]),
			                  std::string(argv[9]) == "left" ? gmres::precond_side::left
			                                                  : gmres::precond_side::right,
			                  std::atoi(argv[10]) != 0};
			auto w = vec::make_device_work<gmres::nwork>(b);
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

	std::FILE * o = std::fopen(argv[2], "wb");
	if (!o)
		return 4;
	int32_t head[3] = {assert_failed ? 100 : static_cast<int32_t>(info.status), info.iters,
	                   info.restarts};
	float norms[5] = {info.res_norm_initial, info.res_norm_final, info.sol_norm_initial,
	                  info.sol_norm_final, info.rhs_norm};
	int64_t nh = static_cast<int64_t>(hist.size());
	std::fwrite(head, sizeof(int32_t), 3, o);
	std::fwrite(norms, sizeof(float), 5, o);
	std::fwrite(&nh, sizeof(int64_t), 1, o);
	std::fwrite(hist.data(), sizeof(double), hist.size(), o);
	const std::vector<double> xo = x.download();
	std::fwrite(xo.data(), sizeof(double), xo.size(), o);
	std::fclose(o);
	fs_csr_destroy(Ah);
	fs_csr_destroy(Dh);
	fs_ctx_destroy(ctx);
	return 0;
}
