// ORACLE -- test infrastructure only.
//
// Runs the reference's own MatrixMarket reader
// (flecsolve/matrices/io/matrix_market.hh) on a file and writes the CSR it
// produces: matrix_market<>::read(file).tocsr() for the whole matrix, and
// definition(file).matrix(range) for a row range.  Built by oracle/Makefile
// against the reference headers plus the stand-ins in oracle/ref_shim/; only
// used to produce the golden fixtures under tests/golden/mm/.
//
// Command line:  ref_mm <file.mtx> <out> [row_begin row_end]
// Output file (little endian): int32 ok (0: the reader threw, nothing else
// follows); int64 nrows, ncols, nnz; int64 rowptr[nrows + 1];
// int64 col[nnz]; double val[nnz]
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <numeric>
#include <vector>

#include "flecsolve/matrices/io/matrix_market.hh"

flecsi::scheduler * flecsi::scheduler::instance = nullptr;

using namespace flecsolve;

namespace {

template<class T>
void wr(std::FILE * f, const T * p, std::size_t n) {
	std::fwrite(p, sizeof(T), n, f);
}

template<class M>
void dump(std::FILE * f, const M & A, std::int64_t nrows, std::int64_t ncols) {
	auto [rowptr, colind, values] = A.rep();
	const std::int64_t nnz = (std::int64_t)rowptr[nrows];
	int ok = 1;
	wr(f, &ok, 1);
	wr(f, &nrows, 1);
	wr(f, &ncols, 1);
	wr(f, &nnz, 1);
	std::vector<std::int64_t> rp(nrows + 1), ci(nnz);
	for (std::int64_t i = 0; i <= nrows; ++i)
		rp[i] = (std::int64_t)rowptr[i];
	for (std::int64_t k = 0; k < nnz; ++k)
		ci[k] = (std::int64_t)colind[k];
	wr(f, rp.data(), rp.size());
	wr(f, ci.data(), ci.size());
	wr(f, &values[0], nnz);
}

} // namespace

int main(int argc, char ** argv) {
	if (argc != 3 && argc != 5) {
		std::fprintf(stderr, "usage: ref_mm <file.mtx> <out> [row_begin row_end]\n");
		return 2;
	}
	std::FILE * f = std::fopen(argv[2], "wb");
	if (!f)
		return 2;
	using mm = mat::io::matrix_market<double>;
	try {
		if (argc == 3) {
			auto A = mm::read(argv[1]).tocsr();
			dump(f, A, (std::int64_t)A.rows(), (std::int64_t)A.cols());
		}
		else {
			mm::definition def(argv[1]);
			std::vector<std::size_t> rng(std::atoll(argv[4]) - std::atoll(argv[3]));
			std::iota(rng.begin(), rng.end(), (std::size_t)std::atoll(argv[3]));
			auto A = def.matrix(rng);
			dump(f, A, (std::int64_t)rng.size(), (std::int64_t)def.num_cols());
		}
	}
	catch (...) {
		int ok = 0;
		wr(f, &ok, 1);
	}
	std::fclose(f);
	return 0;
}
