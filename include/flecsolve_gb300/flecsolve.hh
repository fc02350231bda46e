// flecsolve_gb300/flecsolve.hh -- C++ mirror of flecsolve's Krylov-path API
// over the C ABI of fsgpu.h (header-only; link with -lfsgpu).
//
// Names, argument order and semantics follow the reference so that a caller
// of flecsolve's Krylov path compiles against this header after switching
// the includes:
//
//   vec::device_vec             vec::core<Data, Ops, Config> with the device
//                               Data/Operations policy (flecsolve/vectors/
//                               core.hh:26-353)
//   op::core / op::handle /     flecsolve/operators/{core,handle,shell}.hh
//   op::ref / op::cref / op::I
//   mat::device_csr             mat::csr as an op::base policy
//                               (flecsolve/matrices/seq.hh:35-63)
//   cg / bicgstab / gmres       settings, make_work, nwork, solver(s, w)(A[, P
//                               [, diag]]) -> operator, (b, x) -> solve_info
//                               (flecsolve/solvers/cg.hh:250-270,
//                               bicgstab.hh:193-216, gmres.hh:366-438,
//                               krylov_parameters.hh:94-126)
//   solve_info, solver_settings flecsolve/solvers/solver_settings.hh:31-85
//
// Every call goes to libfsgpu.so; errors become fs_error exceptions, and the
// reference's flog_assert sites (FS_ERR_BREAKDOWN) raise too.
#pragma once

#include <array>
#include <tuple>
#include <cmath>
#include <cstdint>
#include <iterator>
#include <limits>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../fsgpu.h"

namespace flecsolve {

// ------------------------------------------------------------ errors --

struct fs_error : std::runtime_error {
	int status;
	fs_error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(int s, fs_ctx c = nullptr, const char *what = "") {
	if (s != FS_OK) {
		std::string m = std::string(what) + ": " + fs_status_string(s);
		if (c)
			m += std::string(" (") + fs_last_error(c) + ")";
		throw fs_error(s, m);
	}
}

// One device + stream; the FleCSI runtime context of the reference.
class context {
public:
	explicit context(int device = 0) { check(fs_ctx_create(device, &h_), nullptr, "fs_ctx_create"); }
	~context() {
		if (h_)
			fs_ctx_destroy(h_);
	}
	context(const context &) = delete;
	context &operator=(const context &) = delete;
	fs_ctx get() const { return h_; }
	void sync() const { check(fs_ctx_sync(h_), h_, "sync"); }

private:
	fs_ctx h_ = nullptr;
};

// ------------------------------------------------- settings and info ---

// solver_settings.hh:31-36 (float tolerances, as in the reference)
struct solver_settings {
	int maxiter;
	float rtol;
	float atol;
	bool use_zero_guess;
};

// solver_settings.hh:61-85
struct solve_info {
	enum class stop_reason {
		converged_atol,
		converged_rtol,
		converged_user,
		diverged_dtol,
		diverged_iters,
		diverged_breakdown,
		unknown
	};
	stop_reason status = stop_reason::unknown;
	int iters = 0;
	int restarts = 0;
	float res_norm_initial = 0, res_norm_final = 0;
	float sol_norm_initial = 0, sol_norm_final = 0;
	float rhs_norm = 0;
	bool success() const {
		return status == stop_reason::converged_atol || status == stop_reason::converged_rtol ||
		       status == stop_reason::converged_user;
	}
	static solve_info from(const fs_solve_info &i) {
		solve_info o;
		o.status = static_cast<stop_reason>(i.status);
		o.iters = i.iters;
		o.restarts = i.restarts;
		o.res_norm_initial = i.res_norm_initial;
		o.res_norm_final = i.res_norm_final;
		o.sol_norm_initial = i.sol_norm_initial;
		o.sol_norm_final = i.sol_norm_final;
		o.rhs_norm = i.rhs_norm;
		return o;
	}
};

// ----------------------------------------------------------- vectors ---

namespace vec {

// the `.get()` futures of the reference's reductions (util/future.hh)
template<class T>
struct future {
	T val;
	T get() const { return val; }
};

// vec::core over the device Data/Operations policy.  Methods and argument
// order follow flecsolve/vectors/core.hh:59-310 (`this` is the output).
class device_vec {
public:
	using scalar = double;
	using real = double;
	using len_t = std::size_t;

	device_vec(const context &c, std::size_t n) : ctx_(c.get()), owns_(true) {
		check(fs_vec_create(ctx_, (int64_t)n, FS_F64, &h_), ctx_, "fs_vec_create");
	}
	device_vec(const context &c, const std::vector<double> &host) : device_vec(c, host.size()) {
		upload(host);
	}
	// non-owning view of a library vector (the diagnostic's argument)
	static device_vec view(fs_ctx c, fs_vec h) { return device_vec(c, h); }
	// view of n doubles of caller-owned device memory (the handle is freed
	// with the view, the memory is not)
	static device_vec wrap(fs_ctx c, std::size_t n, double *dptr) {
		fs_vec h = nullptr;
		check(fs_vec_wrap(c, (int64_t)n, FS_F64, dptr, &h), c, "fs_vec_wrap");
		device_vec v(c, h);
		v.owns_ = true;
		return v;
	}
	double *device_ptr() const {
		void *p = nullptr;
		check(fs_vec_device_ptr(h_, &p), ctx_, "device_ptr");
		return static_cast<double *>(p);
	}
	device_vec(device_vec &&o) noexcept : ctx_(o.ctx_), h_(o.h_), owns_(o.owns_) { o.h_ = nullptr; }
	device_vec &operator=(device_vec &&o) noexcept {
		std::swap(ctx_, o.ctx_);
		std::swap(h_, o.h_);
		std::swap(owns_, o.owns_);
		return *this;
	}
	device_vec(const device_vec &) = delete;
	~device_vec() {
		if (h_ && owns_)
			fs_vec_destroy(h_);
	}

	fs_vec handle() const { return h_; }
	fs_ctx ctx() const { return ctx_; }

	void upload(const std::vector<double> &host) {
		check(fs_vec_upload(h_, host.data(), (int64_t)host.size()), ctx_, "upload");
	}
	std::vector<double> download() const {
		std::vector<double> out(local_size());
		check(fs_vec_download(h_, out.data(), (int64_t)out.size()), ctx_, "download");
		return out;
	}

	void copy(const device_vec &src) { check(fs_vec_copy(src.h_, h_), ctx_, "copy"); }
	void zero() { check(fs_vec_zero(h_), ctx_, "zero"); }
	void set_scalar(double v) { check(fs_vec_set_scalar(h_, v), ctx_, "set_scalar"); }
	void scale(double a, const device_vec &x) { check(fs_vec_scale(a, x.h_, h_), ctx_, "scale"); }
	void scale(double a) { check(fs_vec_scale_self(a, h_), ctx_, "scale"); }
	void add(const device_vec &x, const device_vec &y) { check(fs_vec_add(x.h_, y.h_, h_), ctx_, "add"); }
	void subtract(const device_vec &x, const device_vec &y) {
		check(fs_vec_subtract(x.h_, y.h_, h_), ctx_, "subtract");
	}
	void multiply(const device_vec &x, const device_vec &y) {
		check(fs_vec_multiply(x.h_, y.h_, h_), ctx_, "multiply");
	}
	void divide(const device_vec &x, const device_vec &y) {
		check(fs_vec_divide(x.h_, y.h_, h_), ctx_, "divide");
	}
	void reciprocal(const device_vec &x) { check(fs_vec_reciprocal(x.h_, h_), ctx_, "reciprocal"); }
	void linear_sum(double a, const device_vec &x, double b, const device_vec &y) {
		check(fs_vec_linear_sum(a, x.h_, b, y.h_, h_), ctx_, "linear_sum");
	}
	void axpy(double a, const device_vec &x, const device_vec &y) {
		check(fs_vec_axpy(a, x.h_, y.h_, h_), ctx_, "axpy");
	}
	void axpby(double a, double b, const device_vec &x) {
		check(fs_vec_axpby(a, b, x.h_, h_), ctx_, "axpby");
	}
	void abs(const device_vec &x) { check(fs_vec_abs(x.h_, h_), ctx_, "abs"); }
	void add_scalar(const device_vec &x, double a) {
		check(fs_vec_add_scalar(x.h_, a, h_), ctx_, "add_scalar");
	}
	void set_random(unsigned seed) { check(fs_vec_set_random(h_, seed), ctx_, "set_random"); }

	future<double> min() const { return red(fs_vec_min); }
	future<double> max() const { return red(fs_vec_max); }
	future<double> l1norm() const { return red(fs_vec_l1norm); }
	future<double> l2norm() const { return red(fs_vec_l2norm); }
	future<double> inf_norm() const { return red(fs_vec_inf_norm); }
	future<double> dot(const device_vec &x) const {
		double r;
		check(fs_vec_dot(h_, x.h_, &r), ctx_, "dot");
		return {r};
	}
	future<std::size_t> global_size() const { return {local_size()}; }
	std::size_t local_size() const {
		int64_t n;
		check(fs_vec_size(h_, &n), ctx_, "size");
		return (std::size_t)n;
	}

private:
	device_vec(fs_ctx c, fs_vec h) : ctx_(c), h_(h), owns_(false) {}
	future<double> red(int (*f)(fs_vec, double *)) const {
		double r;
		check(f(h_, &r), ctx_, "reduction");
		return {r};
	}
	fs_ctx ctx_ = nullptr;
	fs_vec h_ = nullptr;
	bool owns_ = true;
};

// vec::multi (flecsolve/vectors/multi.hh:74-160): components tagged by
// index, stored as views into one contiguous device allocation (`whole()`),
// elementwise ops per component, reductions combined over components the way
// operations/multi.hh:179-253 does (sum of dots, sqrt of summed squares,
// max/min over components, in component order).
class multi {
public:
	multi(const context &c, const std::vector<std::size_t> &sizes)
		: whole_(c, total(sizes)) {
		double *base = whole_.device_ptr();
		std::size_t off = 0;
		for (std::size_t n : sizes) {
			comps_.push_back(device_vec::wrap(c.get(), n, base + off));
			off += n;
		}
	}
	std::size_t size() const { return comps_.size(); }
	device_vec &get(std::size_t i) { return comps_[i]; }
	const device_vec &get(std::size_t i) const { return comps_[i]; }
	device_vec &subset(std::size_t i) { return comps_[i]; }
	device_vec &whole() { return whole_; }
	const device_vec &whole() const { return whole_; }

	template<class F>
	void each(F &&f) {
		for (auto &c : comps_)
			f(c);
	}
	void copy(const multi &s) { zip(s, [](device_vec &a, const device_vec &b) { a.copy(b); }); }
	void zero() { each([](device_vec &c) { c.zero(); }); }
	void set_scalar(double v) { each([v](device_vec &c) { c.set_scalar(v); }); }
	void scale(double a) { each([a](device_vec &c) { c.scale(a); }); }
	void axpy(double a, const multi &x, const multi &y) {
		for (std::size_t i = 0; i < comps_.size(); ++i)
			comps_[i].axpy(a, x.comps_[i], y.comps_[i]);
	}
	future<double> dot(const multi &x) const {
		double s = 0;
		for (std::size_t i = 0; i < comps_.size(); ++i)
			s += comps_[i].dot(x.comps_[i]).get();
		return {s};
	}
	future<double> l2norm() const {
		double s = 0;
		for (auto &c : comps_)
			s += c.dot(c).get();
		return {std::sqrt(s)};
	}
	future<double> l1norm() const {
		double s = 0;
		for (auto &c : comps_)
			s += c.l1norm().get();
		return {s};
	}
	future<double> inf_norm() const { return fold([](const device_vec &c) { return c.inf_norm().get(); }, true); }
	future<double> max() const { return fold([](const device_vec &c) { return c.max().get(); }, true); }
	future<double> min() const { return fold([](const device_vec &c) { return c.min().get(); }, false); }

private:
	static std::size_t total(const std::vector<std::size_t> &s) {
		std::size_t t = 0;
		for (auto n : s)
			t += n;
		return t;
	}
	template<class F>
	void zip(const multi &o, F f) {
		for (std::size_t i = 0; i < comps_.size(); ++i)
			f(comps_[i], o.comps_[i]);
	}
	template<class F>
	future<double> fold(F f, bool is_max) const {
		double r = f(comps_[0]);
		for (std::size_t i = 1; i < comps_.size(); ++i) {
			double v = f(comps_[i]);
			r = is_max ? (v > r ? v : r) : (v < r ? v : r);
		}
		return {r};
	}
	device_vec whole_;
	std::vector<device_vec> comps_;
};

}  // namespace vec

// ---------------------------------------------------------- operators --

namespace op {

// op::base (operators/core.hh:29-78), parameterless form
struct base {};

// op::core<P>: apply / operator() / residual (operators/core.hh:80-143)
template<class P>
struct core : P {
	using P::P;
	core(P p) : P(std::move(p)) {}
	void apply(const vec::device_vec &x, vec::device_vec &y) const { P::apply(x, y); }
	void operator()(const vec::device_vec &x, vec::device_vec &y) const { P::apply(x, y); }
	// r = b - A x
	void residual(const vec::device_vec &b, const vec::device_vec &x, vec::device_vec &r) const {
		P::residual(b, x, r);
	}
};

// op::handle: reference or shared ownership (operators/handle.hh:10-56)
template<class T>
struct handle {
	using type = T;
	std::shared_ptr<T> own;
	T *ptr = nullptr;
	T &get() const { return *ptr; }
};
template<class T>
handle<T> ref(T &o) { return {nullptr, &o}; }
template<class T>
handle<const T> cref(const T &o) { return {nullptr, &o}; }
template<class T, class... A>
handle<T> make_shared(A &&...a) {
	auto p = std::make_shared<T>(std::forward<A>(a)...);
	return {p, p.get()};
}

// op::I, the identity operator (operators/shell.hh:317-318)
struct identity_t {};
inline constexpr identity_t I{};

}  // namespace op

// ------------------------------------------------------------ matrices --

namespace mat {

// The CSR operator on the device.  Constructed from the reference's host CSR
// arrays (std::size_t or int32 column ids, double values).
class device_csr {
public:
	device_csr(const context &c, std::size_t nrows, std::size_t ncols,
	           const std::vector<int64_t> &rowptr, const std::vector<int32_t> &col,
	           const std::vector<double> &val)
		: ctx_(c.get()) {
		check(fs_csr_create(ctx_, (int64_t)nrows, (int64_t)ncols, (int64_t)val.size(), rowptr.data(),
		                    col.data(), 4, val.data(), &h_),
		      ctx_, "fs_csr_create");
	}
	device_csr(const context &c, std::size_t nrows, std::size_t ncols,
	           const std::vector<int64_t> &rowptr, const std::vector<std::size_t> &col,
	           const std::vector<double> &val)
		: ctx_(c.get()) {
		check(fs_csr_create(ctx_, (int64_t)nrows, (int64_t)ncols, (int64_t)val.size(), rowptr.data(),
		                    col.data(), (int)sizeof(std::size_t), val.data(), &h_),
		      ctx_, "fs_csr_create");
	}
	device_csr(device_csr &&o) noexcept : ctx_(o.ctx_), h_(o.h_) { o.h_ = nullptr; }
	// takes ownership of an operator handle the library made (the
	// matrix-free physics operator, physics::op_expr::matrix_free)
	static device_csr adopt(fs_ctx c, fs_csr h) { return device_csr(c, h); }
	// from a host CSR as mat::io::matrix_market produces it
	template<class H, class = decltype(std::declval<const H &>().rowptr)>
	device_csr(const context &c, const H &A) : ctx_(c.get()) {
		check(fs_csr_create(ctx_, (int64_t)A.nrows, (int64_t)A.ncols, (int64_t)A.val.size(),
		                    A.rowptr.data(), A.col.data(), 8, A.val.data(), &h_),
		      ctx_, "fs_csr_create");
	}
	device_csr(const device_csr &) = delete;
	~device_csr() {
		if (h_)
			fs_csr_destroy(h_);
	}
	fs_csr handle() const { return h_; }
	fs_ctx ctx() const { return ctx_; }
	std::size_t rows() const { return shape().first; }
	std::size_t cols() const { return shape().second; }

	// y = A x (mat::sparse::apply -> compressed_ops::spmv)
	void apply(const vec::device_vec &x, vec::device_vec &y) const {
		check(fs_csr_spmv(h_, x.handle(), y.handle(), FS_SPMV_FMA), ctx_, "spmv");
	}
	void residual(const vec::device_vec &b, const vec::device_vec &x, vec::device_vec &r) const {
		check(fs_csr_residual(h_, b.handle(), x.handle(), r.handle()), ctx_, "residual");
	}
	// the D^-1 operator of the reference's tests (util/test/mesh.hh:123-140)
	// as a diagonal vector usable as a preconditioner
	vec::device_vec Dinv(const context &c) const {
		vec::device_vec d(c, rows());
		check(fs_csr_diag_inv(h_, d.handle()), ctx_, "diag_inv");
		return d;
	}

private:
	device_csr(fs_ctx c, fs_csr h) : ctx_(c), h_(h) {}
	std::pair<std::size_t, std::size_t> shape() const {
		int64_t r, c;
		check(fs_csr_shape(h_, &r, &c, nullptr), ctx_, "shape");
		return {(std::size_t)r, (std::size_t)c};
	}
	fs_ctx ctx_;
	fs_csr h_ = nullptr;
};

using csr = op::core<device_csr>;

// Host CSR as the reference's MatrixMarket reader produces it: int64 row
// offsets and global column ids, double values.
struct host_csr {
	std::size_t nrows = 0, ncols = 0;
	std::vector<int64_t> rowptr, col;
	std::vector<double> val;
	std::size_t rows() const { return nrows; }
	std::size_t cols() const { return ncols; }
};

namespace io {

// mat::io::matrix_market (flecsolve/matrices/io/matrix_market.hh:31-183) over
// fs_mm_*: read(file).tocsr() for the whole matrix and definition(file)
// .matrix(range) for a row range, with the reference reader's rules (float
// rounding of values, "symmetric" mirroring, file order within rows).
template<class scalar = double, class size = std::size_t>
struct matrix_market {
	class file {
	public:
		explicit file(const char *fname) {
			const int st = fs_mm_read(fname, &h_);
			if (st != FS_OK)
				throw fs_error(st, std::string("matrix_market: cannot read ") + fname);
		}
		file(file &&o) noexcept : h_(o.h_) { o.h_ = nullptr; }
		file(const file &) = delete;
		~file() {
			if (h_)
				fs_mm_destroy(h_);
		}
		std::size_t num_rows() const { return shape()[0]; }
		std::size_t num_cols() const { return shape()[1]; }
		host_csr rows(std::size_t begin, std::size_t end) const {
			host_csr A;
			A.nrows = end - begin;
			A.ncols = num_cols();
			int64_t nz = 0;
			check(fs_mm_rows(h_, (int64_t)begin, (int64_t)end, nullptr, nullptr, nullptr, &nz), nullptr,
			      "fs_mm_rows");
			A.rowptr.resize(A.nrows + 1);
			A.col.resize((std::size_t)nz);
			A.val.resize((std::size_t)nz);
			check(fs_mm_rows(h_, (int64_t)begin, (int64_t)end, A.rowptr.data(), A.col.data(), A.val.data(),
			                 nullptr),
			      nullptr, "fs_mm_rows");
			return A;
		}
		// coo::tocsr (matrices/seq.hh:324-352) of the whole file
		host_csr tocsr() const { return rows(0, num_rows()); }

	private:
		std::array<int64_t, 2> shape() const {
			int64_t r = 0, c = 0;
			check(fs_mm_shape(h_, &r, &c, nullptr, nullptr), nullptr, "fs_mm_shape");
			return {r, c};
		}
		fs_mm h_ = nullptr;
	};

	// matrix_market::read (matrix_market.hh:64-70)
	static file read(const char *fname) { return file(fname); }

	// matrix_market::definition (matrix_market.hh:103-165)
	struct definition {
		explicit definition(const char *fname) : f(fname) {}
		std::size_t num_rows() const { return f.num_rows(); }
		std::size_t num_cols() const { return f.num_cols(); }
		// rows rng (contiguous), offsets relative to the first, global columns
		template<class Range>
		host_csr matrix(const Range &rng) const {
			return f.rows((std::size_t)*std::begin(rng), (std::size_t)*std::begin(rng) + rng.size());
		}
		file f;
	};
};

}  // namespace io

}  // namespace mat

// --------------------------------------------------------- solvers ----

// default diagnostic (krylov_parameters.hh:29-31)
inline const auto default_diagnostic = [](const vec::device_vec &, double) { return false; };

namespace detail {

struct jacobi_t {};

template<class D>
int diag_trampoline(void *user, fs_vec x, double res) {
	auto *p = static_cast<std::pair<D *, fs_ctx> *>(user);
	auto v = vec::device_vec::view(p->second, x);
	return (*p->first)(v, res) ? 1 : 0;
}

// op::X<krylov_parameters<...>> bound by krylov_solver::operator()
// (krylov_parameters.hh:94-126): owns the device solver and its work.
template<class Diag>
class bound_solver {
public:
	bound_solver(int method, const fs_krylov_settings &s, const mat::csr &A, fs_precond P,
	             Diag diag)
		: ctx_(A.ctx()), diag_(std::make_unique<Diag>(std::move(diag))) {
		check(fs_krylov_create(ctx_, method, &s, A.handle(), &P, &h_), ctx_, "fs_krylov_create");
		if constexpr (!std::is_same_v<std::decay_t<Diag>, std::decay_t<decltype(default_diagnostic)>>) {
			user_ = std::make_unique<std::pair<Diag *, fs_ctx>>(diag_.get(), ctx_);
			check(fs_krylov_set_diagnostic(h_, &diag_trampoline<Diag>, user_.get()), ctx_,
			      "set_diagnostic");
		}
	}
	bound_solver(bound_solver &&) = default;
	~bound_solver() {
		if (h_)
			fs_krylov_destroy(h_);
	}
	// op::core::apply(b, x) -> solve_info
	solve_info apply(const vec::device_vec &b, vec::device_vec &x) const {
		fs_solve_info i{};
		check(fs_krylov_apply(h_, b.handle(), x.handle(), &i), ctx_, "fs_krylov_apply");
		return solve_info::from(i);
	}
	solve_info operator()(const vec::device_vec &b, vec::device_vec &x) const { return apply(b, x); }
	fs_solver handle() const { return h_; }

private:
	fs_ctx ctx_;
	fs_solver h_ = nullptr;
	std::unique_ptr<Diag> diag_;
	std::unique_ptr<std::pair<Diag *, fs_ctx>> user_;
};

inline fs_precond to_precond(op::identity_t) { return {FS_PRECOND_NONE, nullptr, nullptr}; }
inline fs_precond to_precond(jacobi_t) { return {FS_PRECOND_JACOBI, nullptr, nullptr}; }
inline fs_precond to_precond(const vec::device_vec &d) { return {FS_PRECOND_DIAG, d.handle(), nullptr}; }
template<class T>
fs_precond to_precond(const op::handle<T> &h) { return to_precond(h.get()); }

// settings beyond solver_settings (GMRES)
inline void fill_extra(const solver_settings &, fs_krylov_settings &) {}

template<class Settings>
fs_krylov_settings to_c(const Settings &s) {
	fs_krylov_settings k;
	fs_krylov_settings_default(&k);
	k.base.maxiter = s.maxiter;
	k.base.rtol = s.rtol;
	k.base.atol = s.atol;
	k.base.use_zero_guess = s.use_zero_guess ? 1 : 0;
	fill_extra(s, k);
	return k;
}

// work description returned by make_work: the device solver allocates its
// own work vectors from the exemplar's size (solver_settings.hh:189-200)
struct work {
	std::size_t n;
};

// krylov_solver<OpType, Settings, Work> (krylov_parameters.hh:94-126)
template<class Settings, int Method>
struct krylov_solver {
	Settings settings;
	work workspace;

	krylov_solver(Settings s, work w) : settings(std::move(s)), workspace(w) {}

	template<class P = op::identity_t, class D = std::decay_t<decltype(default_diagnostic)>>
	auto operator()(const op::handle<mat::csr> &A, const P &precond = op::I,
	                D diag = default_diagnostic) const {
		return bound_solver<D>(Method, to_c(settings), A.get(), to_precond(precond), std::move(diag));
	}
	template<class P, class D>
	auto operator()(const op::handle<mat::csr> &A, const P &precond,
	                std::reference_wrapper<D> diag) const {
		return bound_solver<std::reference_wrapper<D>>(Method, to_c(settings), A.get(),
		                                               to_precond(precond), diag);
	}
};

}  // namespace detail

// the Jacobi (D^-1) preconditioner computed from A on the device
inline constexpr detail::jacobi_t jacobi{};

// --------------------------------------------------------------- NKA ----
//
// nka::settings / make_work / solver (flecsolve/solvers/nka.hh:514-597) over
// fs_nka_*: solver(settings, work)(A, op::ref(P)) with P a bound Krylov
// solver used as the preconditioner, as solvers/test/nka.cc:72-80 binds it.
namespace nka {
static constexpr std::size_t nwork = 3;  // nka.hh:29
// nka.hh:514-545 with the defaults of nka::options (nka.hh:536-552)
struct settings : solver_settings {
	int max_dim = 0;
	double angle_tol = 0.9;
	int max_fun_evals = 0;
	bool freeze_pc = true;
	bool use_qr = false;
	bool use_damping = false;
	bool adaptive_damping = false;
	double damping_factor = 1.0;
};
template<std::size_t V>
struct dim_bound_t {
	static constexpr std::size_t value = V;
};
template<std::size_t V>
inline constexpr dim_bound_t<V> dim_bound{};
inline detail::work make_work(const vec::device_vec &b) { return {b.local_size()}; }
template<std::size_t V>
detail::work make_work(dim_bound_t<V>, const vec::device_vec &b) {
	return {b.local_size()};
}

// op::core<op::nka<...>>: apply(f, u) -> solve_info
class bound {
public:
	bound(const settings &s, const mat::csr &F, fs_solver P) : ctx_(F.ctx()) {
		fs_nka_settings c;
		fs_nka_settings_default(&c);
		c.base.maxiter = s.maxiter;
		c.base.rtol = s.rtol;
		c.base.atol = s.atol;
		c.base.use_zero_guess = s.use_zero_guess ? 1 : 0;
		c.max_dim = s.max_dim;
		c.angle_tol = s.angle_tol;
		c.max_fun_evals = s.max_fun_evals;
		c.freeze_pc = s.freeze_pc;
		c.use_qr = s.use_qr;
		c.use_damping = s.use_damping;
		c.adaptive_damping = s.adaptive_damping;
		c.damping_factor = s.damping_factor;
		check(fs_nka_create(ctx_, &c, F.handle(), nullptr, nullptr, P, &h_), ctx_, "fs_nka_create");
	}
	bound(bound &&o) noexcept : ctx_(o.ctx_), h_(o.h_) { o.h_ = nullptr; }
	bound(const bound &) = delete;
	~bound() {
		if (h_)
			fs_nka_destroy(h_);
	}
	solve_info apply(const vec::device_vec &f, vec::device_vec &u) const {
		fs_solve_info i{};
		check(fs_nka_apply(h_, f.handle(), u.handle(), &i), ctx_, "fs_nka_apply");
		return solve_info::from(i);
	}
	solve_info operator()(const vec::device_vec &f, vec::device_vec &u) const { return apply(f, u); }

private:
	fs_ctx ctx_;
	fs_nka h_ = nullptr;
};

struct solver {
	settings s;
	detail::work workspace;
	solver(settings st, detail::work w) : s(std::move(st)), workspace(w) {}
	template<class PS>
	bound operator()(const op::handle<mat::csr> &F, const op::handle<PS> &P) const {
		return bound(s, F.get(), P.get().handle());
	}
	bound operator()(const op::handle<mat::csr> &F) const { return bound(s, F.get(), nullptr); }
};
}  // namespace nka

namespace cg {
static constexpr std::size_t nwork = 4;  // cg.hh:252
using settings = solver_settings;        // cg.hh:254
inline detail::work make_work(const vec::device_vec &b) { return {b.local_size()}; }
using solver = detail::krylov_solver<settings, FS_CG>;
}  // namespace cg

namespace bicgstab {
static constexpr std::size_t nwork = 8;  // bicgstab.hh:195
struct settings : solver_settings {};    // bicgstab.hh:197
inline detail::work make_work(const vec::device_vec &b) { return {b.local_size()}; }
using solver = detail::krylov_solver<settings, FS_BICGSTAB>;
}  // namespace bicgstab

namespace gmres {
static constexpr int krylov_dim_bound = 100;                       // gmres.hh:31
static constexpr std::size_t nwork = (krylov_dim_bound + 1) + 3;   // gmres.hh:32
enum class precond_side { left, right };                           // gmres.hh:33
struct settings : solver_settings {                                // gmres.hh:389-405
	int max_krylov_dim;
	precond_side pre_side;
	bool restart;
};
inline detail::work make_work(const vec::device_vec &b) { return {b.local_size()}; }
using solver = detail::krylov_solver<settings, FS_GMRES>;
}  // namespace gmres

namespace gmres {
// found by argument-dependent lookup from detail::to_c
inline void fill_extra(const settings &s, fs_krylov_settings &k) {
	k.max_krylov_dim = s.max_krylov_dim;
	k.pre_side = s.pre_side == precond_side::left ? FS_LEFT : FS_RIGHT;
	k.restart = s.restart ? 1 : 0;
}
}  // namespace gmres

// FP32-inner / FP64-refined variants (no counterpart in the reference)
namespace mixed {
using cg_solver = detail::krylov_solver<cg::settings, FS_CG_MIXED>;
using bicgstab_solver = detail::krylov_solver<bicgstab::settings, FS_BICGSTAB_MIXED>;
using gmres_solver = detail::krylov_solver<gmres::settings, FS_GMRES_MIXED>;
}  // namespace mixed


// ----------------------------------------------------------- physics ----
// The structured-mesh physics operators of flecsolve/physics/ over device
// fields (fs_fvm_* of fsgpu.h).  Spelled as the reference spells them, with
// the mesh passed where the reference takes it from the field's topology:
//   bc<dirichlet, x_axis, boundary_low>::create({1e-9}, m)
//   coefficient<constant_coefficient>::create({1.0}, faces, m)
//   diffusion::create({a, faces, beta, alpha}, m)
//   op_expr(ops...).apply(u, v)  /  op_expr(ops...).matrix_free()
// The operators hold pointers to the mesh and to the fields they were created
// with, which must outlive them; the matrix-free operator copies what it needs
// when it is made.
namespace physics {

enum axis { x_axis = 0, y_axis = 1, z_axis = 2 };
enum domain { boundary_low = 0, boundary_high = 1 };

// fvm_narray with boundary depth 1 on one color (physics/test/
// test_setup.hh:47-74): cells with one boundary layer, faces (n+1)^3 per axis
class fvm_mesh {
public:
	fvm_mesh(const context &c, std::array<int64_t, 3> extents,
	         std::array<std::array<double, 2>, 3> box = {{{0.0, 1.0}, {0.0, 1.0}, {0.0, 1.0}}})
		: ctx_(c.get()) {
		for (int a = 0; a < 3; ++a) {
			m_.n[a] = extents[(std::size_t)a];
			m_.box[a][0] = box[(std::size_t)a][0];
			m_.box[a][1] = box[(std::size_t)a][1];
		}
		check(fs_fvm_geometry(&m_, dx_, dA_, &vol_), ctx_, "fs_fvm_geometry");
	}
	const fs_fvm_mesh &get() const { return m_; }
	fs_ctx ctx() const { return ctx_; }
	std::size_t cells() const { return (std::size_t)((m_.n[0] + 2) * (m_.n[1] + 2) * (m_.n[2] + 2)); }
	std::size_t faces() const { return (std::size_t)((m_.n[0] + 1) * (m_.n[1] + 1) * (m_.n[2] + 1)); }
	std::size_t dofs() const { return (std::size_t)(m_.n[0] * m_.n[1] * m_.n[2]); }
	double dx(axis a) const { return dx_[a]; }
	double normal_dA(axis a) const { return dA_[a]; }
	double volume() const { return vol_; }
	vec::device_vec cell_field(const context &c, double v = 0.0) const {
		vec::device_vec f(c, cells());
		f.set_scalar(v);
		return f;
	}
	std::array<vec::device_vec, 3> face_fields(const context &c, double v = 0.0) const {
		std::array<vec::device_vec, 3> out{vec::device_vec(c, faces()), vec::device_vec(c, faces()),
		                                   vec::device_vec(c, faces())};
		for (auto &f : out)
			f.set_scalar(v);
		return out;
	}
	// the logical cells of a cell field as a vector (i fastest), and back
	void pack(const vec::device_vec &field, vec::device_vec &x) const {
		check(fs_fvm_pack(ctx_, &m_, field.handle(), x.handle()), ctx_, "fs_fvm_pack");
	}
	void unpack(const vec::device_vec &x, vec::device_vec &field) const {
		check(fs_fvm_unpack(ctx_, &m_, x.handle(), field.handle()), ctx_, "fs_fvm_unpack");
	}

private:
	fs_ctx ctx_;
	fs_fvm_mesh m_{};
	double dx_[3], dA_[3], vol_ = 0.0;
};

// operator_parameters<dirichlet<Vec>> / <neumann<Vec>>
// (boundary/dirichlet.hh:35-38, boundary/neumann.hh:31-34)
struct dirichlet {
	double boundary_value = 0.0;
	static constexpr int kind = FS_BC_DIRICHLET;
	double value() const { return boundary_value; }
};
struct neumann {
	double flux_value = 0.0;
	static constexpr int kind = FS_BC_NEUMANN;
	double value() const { return flux_value; }
};

// bc<Spec, Axis, Boundary> (boundary/bc_base.hh:29-57)
template<class Spec, int Axis, int Boundary>
struct bc {
	Spec params;
	const fvm_mesh *m;
	static constexpr int face = 2 * Axis + Boundary;
	static bc create(Spec p, const fvm_mesh &mesh) { return bc{p, &mesh}; }
	void apply(vec::device_vec &u, vec::device_vec &) const {
		check(fs_fvm_boundary(m->ctx(), &m->get(), face, Spec::kind, params.value(), u.handle()), m->ctx(),
		      "fs_fvm_boundary");
	}
};

// operator_parameters<constant_coefficient> / <average_coefficient>
// (volume_diffusion/coefficient.hh:66-71, 119-123)
struct constant_coefficient {
	double coeff_value = 1.0;
};
struct average_coefficient {
	double dummy_value = 1.0;
};

// coefficient<Spec, Vec> (coefficient.hh:47-61): sets the face fields
template<class Spec>
struct coefficient {
	Spec params;
	std::array<vec::device_vec, 3> *faces;
	const fvm_mesh *m;
	static coefficient create(Spec p, std::array<vec::device_vec, 3> &f, const fvm_mesh &mesh) {
		return coefficient{p, &f, &mesh};
	}
	void apply(vec::device_vec &u, vec::device_vec &) const {
		auto &f = *faces;
		if constexpr (std::is_same_v<Spec, average_coefficient>)
			check(fs_fvm_coef_average(m->ctx(), &m->get(), u.handle(), f[0].handle(), f[1].handle(),
			                          f[2].handle()),
			      m->ctx(), "fs_fvm_coef_average");
		else
			check(fs_fvm_coef_constant(m->ctx(), &m->get(), params.coeff_value, f[0].handle(), f[1].handle(),
			                           f[2].handle()),
			      m->ctx(), "fs_fvm_coef_constant");
	}
};

// diffusion<Vec> (volume_diffusion/diffusion.hh:209-250):
// v = -beta div(b grad u) + alpha vol a u on the logical cells
struct diffusion {
	struct params {
		vec::device_vec *a;
		std::array<vec::device_vec, 3> *faces;
		double beta = 1.0, alpha = 0.0;
	};
	params p;
	const fvm_mesh *m;
	static diffusion create(params p, const fvm_mesh &mesh) { return diffusion{p, &mesh}; }
	void apply(vec::device_vec &u, vec::device_vec &v) const {
		auto &f = *p.faces;
		check(fs_fvm_diffusion(m->ctx(), &m->get(), p.beta, p.alpha, p.a->handle(), f[0].handle(),
		                       f[1].handle(), f[2].handle(), u.handle(), v.handle()),
		      m->ctx(), "fs_fvm_diffusion");
	}
};

namespace detail {
// what matrix_free collects from the expression's operators
struct mf_parts {
	fs_fvm_operator_settings s{};
	int nbc = 0, ncoef = 0, ndiff = 0;
	bool constant = false;
	const diffusion *d = nullptr;
};
template<class Spec, int Axis, int Boundary>
void collect(mf_parts &c, const bc<Spec, Axis, Boundary> &o) {
	c.s.bc_kind[o.face] = Spec::kind;
	c.s.bc_value[o.face] = o.params.value();
	++c.nbc;
}
template<class Spec>
void collect(mf_parts &c, const coefficient<Spec> &o) {
	if constexpr (std::is_same_v<Spec, average_coefficient>)
		check(FS_ERR_INVALID_ARG, nullptr, "matrix_free: an average coefficient is nonlinear");
	else {
		c.s.b_value = o.params.coeff_value;
		c.constant = true;
	}
	++c.ncoef;
}
inline void collect(mf_parts &c, const diffusion &o) {
	c.d = &o;
	c.s.beta = o.p.beta;
	c.s.alpha = o.p.alpha;
	++c.ndiff;
}
}  // namespace detail

// op_expr(multivariable<...>, ops...) (expressions/operator_expression.hh:
// 55-143): applies its operators in order
template<class... Ops>
struct op_expr_t {
	std::tuple<Ops...> ops;
	void apply(vec::device_vec &u, vec::device_vec &v) const {
		std::apply([&](const auto &...o) { (o.apply(u, v), ...); }, ops);
	}
	// the expression (one boundary operator per face, at most one constant
	// coefficient setter, one diffusion operator) as an operator on vectors
	// of logical cells for the Krylov solvers
	mat::csr matrix_free() const {
		detail::mf_parts c;
		std::apply([&](const auto &...o) { (detail::collect(c, o), ...); }, ops);
		if (c.nbc != 6 || c.ndiff != 1 || c.ncoef > 1)
			check(FS_ERR_INVALID_ARG, nullptr, "matrix_free: six boundary operators, one diffusion");
		for (int f = 0; f < 6; ++f)
			if (c.s.bc_kind[f] == FS_BC_NONE)
				check(FS_ERR_INVALID_ARG, nullptr, "matrix_free: one boundary operator per face");
		const fvm_mesh *m = c.d->m;
		c.s.mesh = m->get();
		auto &f = *c.d->p.faces;
		fs_csr h = nullptr;
		check(fs_fvm_operator_create(m->ctx(), &c.s, c.d->p.a->handle(), c.constant ? nullptr : f[0].handle(),
		                             c.constant ? nullptr : f[1].handle(), c.constant ? nullptr : f[2].handle(),
		                             &h),
		      m->ctx(), "fs_fvm_operator_create");
		return mat::csr(mat::device_csr::adopt(m->ctx(), h));
	}
};
template<class... Ops>
op_expr_t<Ops...> op_expr(Ops... ops) {
	return {std::tuple<Ops...>(std::move(ops)...)};
}

}  // namespace physics


// ------------------------------------------------- time integrators ----
// time_integrator::bdf (flecsolve/time-integrators/bdf.hh,
// bdf_parameters.hh) over device vectors (fs_bdf_* of fsgpu.h), spelled as
// the reference's test uses it (time-integrators/test/implicit.cc:77-113):
//   bdf::integrator ti(bdf::parameters(s, F, bdf::make_work(x), solver));
//   ti.advance(dt, first_step, x, xnew); ti.check_solution(); ti.update();
//   ti.get_next_dt(good);
// F provides apply_rhs(u, f) and set_scaling(gamma); solver.apply(b, x)
// returns a solve_info.  bdf::linear_integrator keeps the time operator
// I - gamma J of a linear f(u) = J u on the device with a bound Krylov solver.
namespace time_integrator {
namespace bdf {

enum class method { cn, be, bdf2, bdf3, bdf4, bdf5, bdf6 };
enum class predictor { ab2, leapfrog };
enum class strategy { truncation_error, constant, final_constant, limit_relative_change };
enum class controller { H211b, pc4_7, pc11, deadbeat };
enum class error_scaling { fixed_resolution, fixed_scaling };
enum class norm_type { inf, l2, l1 };

// bdf::settings with time_integrator::base_settings (parameters.hh:21-28,
// bdf_parameters.hh:35-55); defaults as bdf::options (bdf_parameters.hh:
// 121-156); the options that have none there must be set
struct settings {
	double initial_time = std::nan(""), final_time = std::nan("");
	int max_steps = -1;
	double max_dt = std::numeric_limits<double>::max();
	double min_dt = std::numeric_limits<double>::min();
	double initial_dt = 0.0;
	bool use_predictor = true, use_initial_predictor = true, has_source_term = false;
	bool combine_timestep_estimators = false;
	bdf::predictor predictor = bdf::predictor::leapfrog;
	bdf::strategy timestep_strategy = bdf::strategy::truncation_error;
	double dt_cut_lower_bound = 0.58754407, dt_growth_upper_bound = 1.702;
	int number_of_time_intervals = 100;
	bdf::method integrator = bdf::method::bdf2, starting_integrator = bdf::method::cn;
	bool calculate_time_trunc_error = false;
	norm_type time_trunc_err_norm = norm_type::inf;
	double target_relative_change = 0.0;
	bool use_pi_controller = true;
	controller pi_controller_type = controller::pc4_7;
	bool control_timestep_variation = false;
	error_scaling time_error_scaling = error_scaling::fixed_scaling;
	double time_rtol = 1e-9, time_atol = 1e-15;
	std::vector<double> problem_scales;

	fs_bdf_settings to_c() const {
		fs_bdf_settings c;
		fs_bdf_settings_default(&c);
		c.initial_time = initial_time;
		c.final_time = final_time;
		c.max_steps = max_steps;
		c.max_dt = max_dt;
		c.min_dt = min_dt;
		c.initial_dt = initial_dt;
		c.use_predictor = use_predictor;
		c.use_initial_predictor = use_initial_predictor;
		c.has_source_term = has_source_term;
		c.combine_timestep_estimators = combine_timestep_estimators;
		c.predictor = (int)predictor;
		c.timestep_strategy = (int)timestep_strategy;
		c.dt_cut_lower_bound = dt_cut_lower_bound;
		c.dt_growth_upper_bound = dt_growth_upper_bound;
		c.number_of_time_intervals = number_of_time_intervals;
		c.integrator = (int)integrator;
		c.starting_integrator = (int)starting_integrator;
		c.calculate_time_trunc_error = calculate_time_trunc_error;
		c.time_trunc_err_norm = (int)time_trunc_err_norm;
		c.target_relative_change = target_relative_change;
		c.use_pi_controller = use_pi_controller;
		c.pi_controller_type = (int)pi_controller_type;
		c.control_timestep_variation = control_timestep_variation;
		c.time_error_scaling = (int)time_error_scaling;
		c.time_rtol = time_rtol;
		c.time_atol = time_atol;
		if (problem_scales.size() > 1)
			check(FS_ERR_UNSUPPORTED, nullptr, "bdf: problem scales of one component");
		c.num_problem_scales = (int)problem_scales.size();
		c.problem_scale = problem_scales.empty() ? 0.0 : problem_scales[0];
		return c;
	}
};

// make_work(x): the integrator allocates its work on the device
struct work {
	fs_ctx ctx;
	std::size_t n;
};
inline work make_work(const vec::device_vec &x) { return {x.ctx(), x.local_size()}; }

template<class O, class S>
struct parameters {
	settings s;
	op::handle<O> F;
	work w;
	op::handle<S> solver;
	parameters(const settings &s, op::handle<O> F, work w, op::handle<S> solver)
		: s(s), F(F), w(w), solver(solver) {}
};

class integrator_base {
public:
	integrator_base(const integrator_base &) = delete;
	~integrator_base() {
		if (h_)
			fs_bdf_destroy(h_);
	}
	void advance(double dt, bool first_step, const vec::device_vec &curr, vec::device_vec &out) {
		check(fs_bdf_advance(h_, dt, first_step ? 1 : 0, curr.handle(), out.handle()), ctx_, "bdf advance");
	}
	bool check_solution() {
		int ok = 0;
		check(fs_bdf_check_solution(h_, &ok), ctx_, "bdf check_solution");
		return ok != 0;
	}
	void update() { check(fs_bdf_update(h_), ctx_, "bdf update"); }
	double get_next_dt(bool good) {
		double dt = 0.0;
		check(fs_bdf_get_next_dt(h_, good ? 1 : 0, &dt), ctx_, "bdf get_next_dt");
		return dt;
	}
	double get_current_time() const { return state().current_time; }
	double get_final_time() const { return state().final_time; }
	double get_current_dt() const { return state().current_dt; }
	int get_current_step() const { return state().current_step; }
	int num_step_rejects() const { return state().num_step_rejects; }
	double get_time_operator_scaling() const { return state().gamma; }

protected:
	integrator_base() = default;
	fs_bdf_state state() const {
		fs_bdf_state st;
		check(fs_bdf_state_get(h_, &st), ctx_, "bdf state");
		return st;
	}
	fs_ctx ctx_ = nullptr;
	fs_bdf h_ = nullptr;
};

// bdf::integrator(bdf::parameters(s, F, make_work(x), solver))
template<class O, class S>
class integrator : public integrator_base {
public:
	explicit integrator(parameters<O, S> p) : p_(std::make_unique<parameters<O, S>>(std::move(p))) {
		ctx_ = p_->w.ctx;
		fs_bdf_settings c = p_->s.to_c();
		check(fs_bdf_create(ctx_, &c, (int64_t)p_->w.n, &rhs_tr, p_.get(), &solve_tr, p_.get(), &h_), ctx_,
		      "fs_bdf_create");
	}

private:
	static int rhs_tr(void *user, fs_vec u, fs_vec f) {
		auto *p = static_cast<parameters<O, S> *>(user);
		try {
			auto U = vec::device_vec::view(p->w.ctx, u), Fv = vec::device_vec::view(p->w.ctx, f);
			p->F.get().apply_rhs(U, Fv);
			return FS_OK;
		}
		catch (...) {
			return FS_ERR_INVALID_ARG;
		}
	}
	static int solve_tr(void *user, double gamma, fs_vec b, fs_vec x, int *success) {
		auto *p = static_cast<parameters<O, S> *>(user);
		try {
			p->F.get().set_scaling(gamma);
			auto B = vec::device_vec::view(p->w.ctx, b), X = vec::device_vec::view(p->w.ctx, x);
			solve_info info = p->solver.get().apply(B, X);
			*success = info.success() ? 1 : 0;
			return FS_OK;
		}
		catch (...) {
			return FS_ERR_INVALID_ARG;
		}
	}
	std::unique_ptr<parameters<O, S>> p_;
};
template<class O, class S>
integrator(parameters<O, S>) -> integrator<O, S>;

// f(u) = J u with the time operator I - gamma J on the device, solved by a
// Krylov solver bound to it (method FS_CG ... FS_GMRES_MIXED); J is read at
// every step and must outlive the integrator
class linear_integrator : public integrator_base {
public:
	linear_integrator(const settings &s, const mat::csr &J, int method, const fs_krylov_settings &ks,
	                  bool jacobi = false) {
		ctx_ = J.ctx();
		fs_bdf_settings c = s.to_c();
		fs_precond P{jacobi ? FS_PRECOND_JACOBI : FS_PRECOND_NONE, nullptr, nullptr};
		check(fs_bdf_create_linear(ctx_, &c, J.handle(), method, &ks, &P, &h_), ctx_, "fs_bdf_create_linear");
	}
};

}  // namespace bdf
}  // namespace time_integrator

}  // namespace flecsolve
