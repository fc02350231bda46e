// Stand-in for the part of FleCSI's structured-mesh topology (topo::narray)
// that flecsolve's finite-volume physics operators (flecsolve/physics/) use,
// for one color on one process.  The specialization's own interface
// (physics/specializations/fvm_narray.hh: ranges, spacing, areas, volume) and
// the operator tasks are the reference's code; this file only supplies the
// index layout they are written against:
//  * cells: per axis a boundary layer of depth 1 on each side, so n logical
//    cells [1, n] inside [0, n + 1] (hdepth = bdepth = 1, one color);
//  * faces: an auxiliary index space (bdepth 0) with n + 1 entities per
//    axis, all logical, face i lying between cells i and i + 1;
//  * a field is a dense [k][j][i] array over its space's full extents,
//    i fastest (the mdspan the tasks index).
#pragma once
#include <array>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "flecsi/execution.hh"
#include "flecsi/util/array_ref.hh"
#include "flecsi/util/constant.hh"

#ifndef FLECSI_INLINE_TARGET
#define FLECSI_INLINE_TARGET inline
#endif

namespace flecsi::topo {

template<auto S, class R>
constexpr R make_ids(R r) { return r; }

struct narray_base {
	enum domain { logical, extended, all, boundary_low, boundary_high, ghost_low, ghost_high, global };
	using coord = std::vector<std::size_t>;
	using gcoord = std::vector<util::gid>;
	using colors = std::vector<std::size_t>;
	using hypercube = std::array<coord, 2>;
	struct axis_definition {
		std::size_t hdepth = 0, bdepth = 0;
		bool auxiliary = false;
	};
	struct index_definition {
		std::vector<axis_definition> axes;
	};
	struct coloring {
		std::vector<index_definition> idx_colorings;
	};
	static std::vector<std::size_t> distribute(std::size_t, std::vector<util::gid>) { return {}; }
};

template<class P>
struct narray {
	using base = narray_base;
};

// a field accessor: the field's storage
struct field_view {
	double * p = nullptr;
};

// [k][j][i] view of a field over a space with extents nx, ny (and nz)
struct box_view {
	double * p;
	std::size_t ny, nx;
	struct plane {
		double * p;
		std::size_t nx;
		double * operator[](std::size_t j) const { return p + j * nx; }
	};
	plane operator[](std::size_t k) const { return {p + k * ny * nx, nx}; }
};

// the topology accessor's base: axis layouts, policy metadata, mdspan
template<class D>
struct narray_accessor {
	std::array<std::size_t, 3> n{{1, 1, 1}};  // logical cells per axis (x, y, z)
	typename D::meta_data meta{};

	struct layout_t {
		std::size_t ext0, log0, log1, ext1;
		std::size_t extent() const { return ext1 - ext0; }
		util::iota_view<std::size_t> logical() const { return {log0, log1}; }
		util::iota_view<std::size_t> all() const { return {ext0, ext1}; }
		template<int S>
		std::size_t logical() const { return S == 0 ? log0 : log1; }
		template<int S>
		std::size_t extended() const { return S == 0 ? ext0 : ext1; }
	};
	struct axis_t {
		layout_t layout;
		std::size_t global_id(std::size_t i) const { return i; }
	};

	template<auto Space, auto A>
	axis_t axis() const {
		const std::size_t na = n[(std::size_t)A];
		if (Space == D::cells)
			return {{0, 1, na + 1, na + 2}};
		return {{0, 0, na + 1, na + 1}};
	}
	template<auto A>
	static constexpr std::uint32_t to_idx() { return (std::uint32_t)A; }
	typename D::meta_data & policy_meta() { return meta; }

	template<auto Space>
	std::array<std::size_t, 3> extents() const {
		const std::size_t e = Space == D::cells ? 2 : 1;
		return {{n[0] + e, n[1] + e, n[2] + e}};
	}
	template<auto Space>
	box_view mdspan(field_view f) const {
		const auto e = extents<Space>();
		return {f.p, e[1], e[0]};
	}
};

template<template<class> class C, class D>
struct specialization {
	using base = typename C<D>::base;
	template<auto... V>
	using has = util::constants<V...>;
	template<privilege P>
	struct accessor : D::template interface<narray_accessor<D>> {};
	struct topology {};
	using ptr = topology *;
};

} // namespace flecsi::topo
