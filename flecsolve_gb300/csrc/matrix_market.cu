// MatrixMarket coordinate files, read the way the reference reads them.
//
// Host code only (no device work): the input side of the CSR operator.  The
// reference's reader (flecsolve/matrices/io/matrix_market.hh:31-183) fills a
// COO matrix and converts it with coo::tocsr (matrices/seq.hh:324-352); its
// callers build mat::csr / mat::parcsr operators from the result.  This
// reader produces the same CSR, entry for entry and bit for bit, and rejects
// the files the reference's reader throws on:
//  * header: every line up to and including the first one that does not start
//    with '%'; a "symmetric" anywhere in those lines (also in
//    "skew-symmetric" or in a comment) mirrors the entries; the first
//    non-comment line gives rows, columns and entries as the atoi of its
//    first three ' '-separated fields (a missing field counts 0);
//  * entries: the next `entries` lines, each three ' '-separated fields
//    "row col value" read with std::stoi / std::stoi / std::stof into one
//    string (a missing field repeats the previous one), so a value is
//    rounded to float and then widened to double, and a field that stoi /
//    stof rejects (empty, not a number, out of the float range) fails the
//    read; with mirroring, an off-diagonal entry is followed by its
//    transpose with the same value;
//  * CSR: entries stably sorted by row, so a row keeps the file order of its
//    entries, duplicates included.
// Row or column ids outside the matrix fail the read (the reference has no
// check there).  A row range is cut as the reference's definition::matrix
// does (matrix_market.hh:126-156): offsets relative to the range's first
// entry, global column ids.
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fsgpu_internal.cuh"

namespace fsg {

namespace {

constexpr int kMagicMm = 0x46534D4D;  // 'FSMM'

struct Mm {
	int magic = kMagicMm;
	int64_t nrows = 0, ncols = 0, entries = 0;
	bool symmetric = false;
	std::vector<int64_t> rowptr, col;
	std::vector<double> val;
};

bool ok_mm(const Mm *m) { return m && m->magic == kMagicMm; }

// the first three ' '-separated fields of the size line, atoi'd
void header_sizes(const std::string &line, int64_t (&sz)[3]) {
	std::istringstream in(line);
	for (int i = 0; i < 3; ++i) {
		std::string field;
		std::getline(in, field, ' ');
		sz[i] = std::atoi(field.c_str());
	}
}

// One entry line; false where the reference's stoi / stof throw.  The three
// fields are read into one string, as the reference does: a read past the end
// of the line leaves the previous field in it, so a line with only "row col"
// (a pattern file) reads the column field again as the value.
bool entry(const std::string &line, long long &r, long long &c, double &v) {
	std::istringstream in(line);
	std::string field;
	try {
		std::getline(in, field, ' ');
		r = (long long)std::stoi(field) - 1;
		std::getline(in, field, ' ');
		c = (long long)std::stoi(field) - 1;
		std::getline(in, field, ' ');
		v = (double)std::stof(field);
	}
	catch (...) {
		return false;
	}
	return true;
}

int read_file(const char *path, Mm &m) {
	std::ifstream fh(path);
	if (!fh)
		return FS_ERR_IO;
	std::string line;
	bool sized = false;
	int64_t sz[3] = {0, 0, 0};
	while (std::getline(fh, line)) {
		if (line.find("symmetric") != std::string::npos)
			m.symmetric = true;
		if (line.empty() || line[0] != '%') {
			header_sizes(line, sz);
			sized = true;
			break;
		}
	}
	if (!sized || sz[0] < 0 || sz[1] < 0 || sz[2] < 0)
		return FS_ERR_IO;
	m.nrows = sz[0];
	m.ncols = sz[1];
	m.entries = sz[2];
	const size_t reserve = (size_t)(m.symmetric ? 2 * m.entries : m.entries);
	std::vector<long long> I, J;
	std::vector<double> V;
	I.reserve(reserve);
	J.reserve(reserve);
	V.reserve(reserve);
	for (int64_t k = 0; k < m.entries; ++k) {
		if (!std::getline(fh, line))
			line.clear();
		long long r, c;
		double v;
		if (!entry(line, r, c, v) || r < 0 || r >= m.nrows || c < 0 || c >= m.ncols)
			return FS_ERR_IO;
		I.push_back(r);
		J.push_back(c);
		V.push_back(v);
		if (m.symmetric && r != c) {
			if (c >= m.nrows || r >= m.ncols)
				return FS_ERR_IO;
			I.push_back(c);
			J.push_back(r);
			V.push_back(v);
		}
	}
	// stable counting sort by row
	const size_t nz = V.size();
	m.rowptr.assign((size_t)m.nrows + 1, 0);
	for (size_t k = 0; k < nz; ++k)
		m.rowptr[(size_t)I[k] + 1]++;
	for (int64_t i = 0; i < m.nrows; ++i)
		m.rowptr[(size_t)i + 1] += m.rowptr[(size_t)i];
	std::vector<int64_t> fill(m.rowptr.begin(), m.rowptr.end() - 1);
	m.col.resize(nz);
	m.val.resize(nz);
	for (size_t k = 0; k < nz; ++k) {
		const int64_t slot = fill[(size_t)I[k]]++;
		m.col[(size_t)slot] = J[k];
		m.val[(size_t)slot] = V[k];
	}
	return FS_OK;
}

}  // namespace

}  // namespace fsg

using namespace fsg;

extern "C" {

FS_API int fs_mm_read(const char *path, fs_mm *out) {
	if (!path || !out)
		return FS_ERR_INVALID_ARG;
	*out = nullptr;
	Mm *m = new Mm();
	int st;
	try {
		st = read_file(path, *m);
	}
	catch (...) {
		st = FS_ERR_IO;
	}
	if (st != FS_OK) {
		delete m;
		return st;
	}
	*out = reinterpret_cast<fs_mm>(m);
	return FS_OK;
}

FS_API int fs_mm_shape(fs_mm h, int64_t *nrows, int64_t *ncols, int64_t *nnz, int *symmetric) {
	const Mm *m = reinterpret_cast<const Mm *>(h);
	if (!ok_mm(m))
		return FS_ERR_BAD_HANDLE;
	if (nrows)
		*nrows = m->nrows;
	if (ncols)
		*ncols = m->ncols;
	if (nnz)
		*nnz = (int64_t)m->val.size();
	if (symmetric)
		*symmetric = m->symmetric ? 1 : 0;
	return FS_OK;
}

FS_API int fs_mm_rows(fs_mm h, int64_t row_begin, int64_t row_end, int64_t *rowptr, int64_t *col,
                      double *val, int64_t *nnz_out) {
	const Mm *m = reinterpret_cast<const Mm *>(h);
	if (!ok_mm(m))
		return FS_ERR_BAD_HANDLE;
	if (row_begin < 0 || row_end < row_begin || row_end > m->nrows)
		return FS_ERR_INVALID_ARG;
	const int64_t k0 = m->rowptr[(size_t)row_begin], k1 = m->rowptr[(size_t)row_end];
	if (nnz_out)
		*nnz_out = k1 - k0;
	if (rowptr)
		for (int64_t i = row_begin; i <= row_end; ++i)
			rowptr[i - row_begin] = m->rowptr[(size_t)i] - k0;
	if (col)
		for (int64_t k = k0; k < k1; ++k)
			col[k - k0] = m->col[(size_t)k];
	if (val)
		for (int64_t k = k0; k < k1; ++k)
			val[k - k0] = m->val[(size_t)k];
	return FS_OK;
}

FS_API int fs_mm_destroy(fs_mm h) {
	Mm *m = reinterpret_cast<Mm *>(h);
	if (!ok_mm(m))
		return FS_ERR_BAD_HANDLE;
	m->magic = 0;
	delete m;
	return FS_OK;
}

}  // extern "C"
