// Maintainer-side binding of libfsgpu.so under flecsolve's own templates.
//
// Include this after (or instead of) flecsolve/vectors/seq.hh in a program
// built against a flecsolve checkout: it adds a device Data/Operations policy
// pair for vec::core (flecsolve/vectors/core.hh:25-350, the same policy
// shape as seq_data / seq_ops, vectors/seq.hh:29-305, and topo_view,
// vectors/data/topo_view.hh:23-71 + operations/topo_view.hh:26-291) and a
// device CSR operator policy for op::core (operators/core.hh:29-143).  With
// them, every generic flecsolve solver (cg.hh, the flexible CG, bicgstab.hh,
// gmres.hh, nka.hh) runs unchanged on device vectors: each vector operation
// is one kernel of the library, each reduction's `.get()` one host read of a
// deterministic device reduction, each operator application one device SpMV
// (or whatever a user's op::make_shell does with device vectors).
//
// Everything goes through the C ABI of include/fsgpu.h.  Status codes other
// than FS_OK become flog_assert failures, where the reference asserts.
//
// The fused device loops (one CUDA graph per k iterations, no host read per
// reduction) are reached through fs_krylov_* instead; include/flecsolve_gb300/
// flecsolve.hh mirrors them with the reference's names.
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

#include "fsgpu.h"

#include "flecsi/flog.hh"
#include "flecsolve/operators/core.hh"
#include "flecsolve/vectors/core.hh"
#include "flecsolve/vectors/variable.hh"

namespace flecsolve::vec {

inline void device_check(int status) {
	flog_assert(status == FS_OK, fs_status_string(status));
}

// Config of a device vector (the seq_config of vectors/seq.hh:29-38): real
// FP64 scalars, one component.
template<class Scalar = double, auto V = anon_var::anonymous>
struct device_config {
	static_assert(std::is_same_v<Scalar, double>, "device vectors hold FP64 values");
	using scalar = Scalar;
	using real = Scalar;
	static constexpr bool is_complex = false;
	using len_t = std::size_t;
	static constexpr auto var = variable<V>;
	using var_t = decltype(V);
	static constexpr std::size_t num_components = 1;
};

// Data: an owned device vector of the library (fs_vec) on a context.  A copy
// is a deep copy, as a copy of seq_data's std::vector is.
template<class Config>
struct device_data {
	using config = Config;
	using scalar = typename Config::scalar;
	using size_type = typename Config::len_t;

	device_data() = default;
	device_data(fs_ctx c, size_type n) : ctx(c) { create(n); }
	device_data(const device_data & o) : ctx(o.ctx) {
		if (o.h) {
			create(o.size());
			device_check(fs_vec_copy(o.h, h));
		}
	}
	device_data(device_data && o) noexcept : ctx(o.ctx), h(std::exchange(o.h, nullptr)) {}
	device_data & operator=(const device_data & o) {
		if (this != &o) {
			if (!o.h) {
				release();
				ctx = o.ctx;
				return *this;
			}
			ctx = o.ctx;
			resize(o.size());
			device_check(fs_vec_copy(o.h, h));
		}
		return *this;
	}
	device_data & operator=(device_data && o) noexcept {
		if (this != &o) {
			release();
			ctx = o.ctx;
			h = std::exchange(o.h, nullptr);
		}
		return *this;
	}
	~device_data() { release(); }

	size_type size() const {
		int64_t n = 0;
		if (h)
			device_check(fs_vec_size(h, &n));
		return static_cast<size_type>(n);
	}
	void resize(size_type n) {
		if (h && size() == n)
			return;
		release();
		create(n);
	}

	fs_ctx ctx = nullptr;
	fs_vec h = nullptr;

private:
	void create(size_type n) {
		flog_assert(ctx != nullptr, "device vector without a context");
		device_check(fs_vec_create(ctx, static_cast<int64_t>(n), FS_F64, &h));
	}
	void release() {
		if (h)
			fs_vec_destroy(h);
		h = nullptr;
	}
};

// Operations (the static policy of seq_ops, vectors/seq.hh:69-305): one C ABI
// call each, the same argument meaning (the last argument is `this`).
template<class Data>
struct device_ops {
	using config = typename Data::config;
	using scalar = typename config::scalar;
	using real = typename config::real;
	static constexpr bool is_complex = false;
	using len_t = typename config::len_t;

	// a reduction's result: the value is on the host once the call returns
	template<class T>
	struct fut {
		fut(T v) : val{v} {}
		T val;
		T get() const { return val; }
	};

	static void copy(const Data & src, Data & dest) {
		if (dest.ctx == nullptr)
			dest.ctx = src.ctx;
		dest.resize(src.size());
		device_check(fs_vec_copy(src.h, dest.h));
	}
	static void zero(Data & x) { device_check(fs_vec_zero(x.h)); }
	static void set_random(Data & x, unsigned seed) { device_check(fs_vec_set_random(x.h, seed)); }
	static void set_to_scalar(scalar a, Data & x) { device_check(fs_vec_set_scalar(x.h, a)); }
	static void scale(scalar a, Data & x) { device_check(fs_vec_scale_self(a, x.h)); }
	static void scale(scalar a, const Data & x, Data & y) { device_check(fs_vec_scale(a, x.h, y.h)); }
	static void add(const Data & x, const Data & y, Data & z) { device_check(fs_vec_add(x.h, y.h, z.h)); }
	static void subtract(const Data & x, const Data & y, Data & z) {
		device_check(fs_vec_subtract(x.h, y.h, z.h));
	}
	static void multiply(const Data & x, const Data & y, Data & z) {
		device_check(fs_vec_multiply(x.h, y.h, z.h));
	}
	static void divide(const Data & x, const Data & y, Data & z) {
		device_check(fs_vec_divide(x.h, y.h, z.h));
	}
	static void reciprocal(const Data & x, Data & y) { device_check(fs_vec_reciprocal(x.h, y.h)); }
	static void linear_sum(scalar a, const Data & x, scalar b, const Data & y, Data & z) {
		device_check(fs_vec_linear_sum(a, x.h, b, y.h, z.h));
	}
	static void axpy(scalar a, const Data & x, const Data & y, Data & z) {
		device_check(fs_vec_axpy(a, x.h, y.h, z.h));
	}
	static void axpby(scalar a, scalar b, const Data & x, Data & z) {
		device_check(fs_vec_axpby(a, b, x.h, z.h));
	}
	static void abs(const Data & x, Data & y) { device_check(fs_vec_abs(x.h, y.h)); }
	static void add_scalar(const Data & x, scalar a, Data & y) {
		device_check(fs_vec_add_scalar(x.h, a, y.h));
	}
	static void dump(std::string_view pre, const Data & x) {
		std::vector<double> v(x.size());
		device_check(fs_vec_download(x.h, v.data(), static_cast<int64_t>(v.size())));
		std::FILE * f = std::fopen(std::string(pre).c_str(), "w");
		if (!f)
			return;
		for (double d : v)
			std::fprintf(f, "%.17g\n", d);
		std::fclose(f);
	}
	static fut<real> min(const Data & x) { return reduce(fs_vec_min, x); }
	static fut<real> max(const Data & x) { return reduce(fs_vec_max, x); }
	template<unsigned short p>
	static fut<real> lp_norm(const Data & x) {
		static_assert(p == 1 || p == 2, "device vectors provide the l1 and l2 norms");
		return reduce(p == 1 ? fs_vec_l1norm : fs_vec_l2norm, x);
	}
	static fut<real> inf_norm(const Data & x) { return reduce(fs_vec_inf_norm, x); }
	static fut<scalar> dot(const Data & x, const Data & y) {
		double r = 0;
		device_check(fs_vec_dot(x.h, y.h, &r));
		return r;
	}
	static len_t local_size(const Data & x) { return x.size(); }
	static fut<len_t> global_size(const Data & x) { return local_size(x); }

private:
	static fut<real> reduce(int (*f)(fs_vec, double *), const Data & x) {
		double r = 0;
		device_check(f(x.h, &r));
		return r;
	}
};

template<class T = double, auto V = anon_var::anonymous>
struct device_vec : core<device_data, device_ops, device_config<T, V>> {
	using base = core<device_data, device_ops, device_config<T, V>>;
	using data_type = device_data<device_config<T, V>>;
	device_vec() : base{data_type{}} {}
	device_vec(fs_ctx ctx, std::size_t n) : base{data_type{ctx, n}} {}
	device_vec(variable_t<V>, fs_ctx ctx, std::size_t n) : base{data_type{ctx, n}} {}

	void upload(const std::vector<double> & host) {
		device_check(fs_vec_upload(this->data.h, host.data(), static_cast<int64_t>(host.size())));
	}
	std::vector<double> download() const {
		std::vector<double> host(this->data.size());
		device_check(fs_vec_download(this->data.h, host.data(), static_cast<int64_t>(host.size())));
		return host;
	}
};

// Work vectors shaped like `exemplar` (the role of the reference's
// work_factory / seq_work, solvers/solver_settings.hh:123-200)
template<std::size_t N, class T, auto V>
std::array<device_vec<T, V>, N> make_device_work(const device_vec<T, V> & exemplar) {
	std::array<device_vec<T, V>, N> w;
	for (auto & v : w) {
		v.data.ctx = exemplar.data.ctx;
		v.data.resize(exemplar.data.size());
	}
	return w;
}

} // namespace flecsolve::vec

namespace flecsolve::mat {

// A device CSR operator policy: op::core<device_csr> applies y = A x with the
// reference's row arithmetic (matrices/seq.hh:177-193, products rounded and
// summed left to right).  The handle belongs to the caller.
struct device_csr : op::base<> {
	explicit device_csr(fs_csr A) : h(A) {}

	template<class D, class R>
	void apply(const D & x, R & y) const {
		vec::device_check(fs_csr_spmv(h, x.data.h, y.data.h, FS_SPMV_EXACT));
	}

	fs_csr h;
};

} // namespace flecsolve::mat
