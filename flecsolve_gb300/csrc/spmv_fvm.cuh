// Matrix-free finite-volume diffusion operator, applied where the solvers
// apply a matrix.
//
// The operator is the reference's volume diffusion with its boundary
// operators (flecsolve/physics/volume_diffusion/diffusion.hh:109-193,
// physics/boundary/dirichlet.hh:49-63, physics/boundary/neumann.hh:49-74):
//   v = -beta div(b grad u) + alpha vol a u
// on the logical cells of an nx x ny x nz mesh, written as the sum of face
// fluxes  f = t (u_hi - u_lo),  t = b (dA / dx)  per face.  A vector holds
// the logical cells only (r = i + nx (j + ny k), the order of the reference
// vectors' degrees of freedom); the boundary layer is not stored: a
// neighbour outside the mesh is the ghost value the boundary operator would
// have written, the Dirichlet value or, for a Neumann face, the cell's own
// value minus (nd dx) q.  Per cell the kernel evaluates the same IEEE
// operations in the same order as the reference's three tasks (flux, surface
// sum, volume term), so v is identical bit for bit to the reference's apply
// on a field with those boundary values.
//
// Face transmissibilities t are stored per axis in the reference's face
// layout ((nz+1) x (ny+1) x (nx+1), [k][j][i], face i between cells i and
// i + 1 of the padded cell index), or are one constant per axis.  One thread
// per cell of a 256-cell segment of an x line, segments strided over a
// persistent grid: neighbouring lines and planes are re-read from L1/L2, so
// a sweep reads u, the three face arrays and a (when stored) about once.
#pragma once

namespace fsg {

constexpr int kFvmThreads = 256;

// face order of the boundary arrays: x low, x high, y low, y high, z low,
// z high
enum { kFvmBcNone = 0, kFvmBcDirichlet = 1, kFvmBcNeumann = 2 };

template<class V>
struct FvmDev {
	const V *__restrict__ t[3];  // per axis face transmissibilities, or null
	V tc[3];                     // ... the constant ones
	const V *__restrict__ av;    // (alpha vol) a per logical cell, or null
	V avc;                       // ... the constant
	V neg_beta;                  // -beta
	V ghost_val[6];              // Dirichlet: the value; Neumann: the shift
	int ghost_kind[6];
	int nx, ny, nz;
};

struct FvmOp {
	int nx = 0, ny = 0, nz = 0;
	double beta = 1.0, alpha = 0.0;
	double dx[3] = {1, 1, 1}, dA[3] = {1, 1, 1}, vol = 1.0, c[3] = {1, 1, 1};  // c = dA / dx
	int bc_kind[6] = {0, 0, 0, 0, 0, 0};
	double bc_value[6] = {0, 0, 0, 0, 0, 0};
	double ghost[6] = {0, 0, 0, 0, 0, 0};  // Dirichlet value or Neumann shift (nd dx) q
	double tc[3] = {0, 0, 0};              // constant transmissibilities
	double avc = 0.0;                      // constant (alpha vol) a
	double *t64[3] = {nullptr, nullptr, nullptr};
	float *t32[3] = {nullptr, nullptr, nullptr};
	double *av64 = nullptr;
	float *av32 = nullptr;
	bool affine = false;  // a boundary term that does not vanish at u = 0
	template<class V>
	FvmDev<V> dev() const {
		FvmDev<V> d;
		for (int a = 0; a < 3; ++a) {
			if constexpr (sizeof(V) == 8)
				d.t[a] = t64[a];
			else
				d.t[a] = t32[a];
			d.tc[a] = (V)tc[a];
		}
		if constexpr (sizeof(V) == 8)
			d.av = av64;
		else
			d.av = av32;
		d.avc = (V)avc;
		d.neg_beta = (V)(-beta);
		for (int f = 0; f < 6; ++f) {
			d.ghost_kind[f] = bc_kind[f];
			d.ghost_val[f] = (V)ghost[f];
		}
		d.nx = nx;
		d.ny = ny;
		d.nz = nz;
		return d;
	}
};

// the value of the boundary cell beyond face f of a cell whose value is u
template<class V>
__device__ __forceinline__ V fvm_ghost(const FvmDev<V> &A, int f, V u) {
	return A.ghost_kind[f] == kFvmBcDirichlet ? A.ghost_val[f] : sub_rn(u, A.ghost_val[f]);
}

template<class V, bool TF>
__device__ __forceinline__ V fvm_t(const FvmDev<V> &A, int axis, int idx) {
	if constexpr (TF)
		return __ldg(A.t[axis] + idx);
	else
		return A.tc[axis];
}

// v at logical cell (i, j, k), r its index, with u read through the gather.
// TF: face transmissibility fields (else constants); AV: a cell field of
// (alpha vol) a (else a constant).  Indices fit in int (the cell field of the
// mesh has fewer than 2^31 entries).
template<class V, bool TF, bool AV, class G>
__device__ __forceinline__ V fvm_cell(const FvmDev<V> &A, const G &g, int i, int j, int k, int r) {
	const int nx = A.nx, ny = A.ny, nz = A.nz;
	const int fx = nx + 1, fxy = fx * (ny + 1), plane = nx * ny;
	const V uc = g.at(r);
	const V uw = i > 0 ? g.at(r - 1) : fvm_ghost(A, 0, uc);
	const V ue = i + 1 < nx ? g.at(r + 1) : fvm_ghost(A, 1, uc);
	const V us = j > 0 ? g.at(r - nx) : fvm_ghost(A, 2, uc);
	const V un = j + 1 < ny ? g.at(r + nx) : fvm_ghost(A, 3, uc);
	const V ud = k > 0 ? g.at(r - plane) : fvm_ghost(A, 4, uc);
	const V uu = k + 1 < nz ? g.at(r + plane) : fvm_ghost(A, 5, uc);
	// face indices in the padded face layout; the cell is (i+1, j+1, k+1)
	const int ix = ((k + 1) * (ny + 1) + (j + 1)) * fx + i;  // x face i, low
	const int iy = ix + 1 - fx;                               // y face j, low
	const int iz = ix + 1 - fxy;                              // z face k, low
	const V fx_hi = mul_rn(fvm_t<V, TF>(A, 0, ix + 1), sub_rn(ue, uc));
	const V fx_lo = mul_rn(fvm_t<V, TF>(A, 0, ix), sub_rn(uc, uw));
	const V fy_hi = mul_rn(fvm_t<V, TF>(A, 1, iy + fx), sub_rn(un, uc));
	const V fy_lo = mul_rn(fvm_t<V, TF>(A, 1, iy), sub_rn(uc, us));
	const V fz_hi = mul_rn(fvm_t<V, TF>(A, 2, iz + fxy), sub_rn(uu, uc));
	const V fz_lo = mul_rn(fvm_t<V, TF>(A, 2, iz), sub_rn(uc, ud));
	const V du = add_rn(add_rn(sub_rn(fx_hi, fx_lo), sub_rn(fy_hi, fy_lo)), sub_rn(fz_hi, fz_lo));
	V av;
	if constexpr (AV)
		av = __ldg(A.av + r);
	else
		av = A.avc;
	return add_rn(mul_rn(A.neg_beta, du), mul_rn(av, uc));
}

// One thread per cell of a 256-cell segment of an x line; CTAs stride over
// the segments, the (segment, j, k) position advanced by additions only.
template<class V, bool TF, bool AV, class G, class Epi>
__global__ void __launch_bounds__(kFvmThreads)
spmv_fvm_kernel(FvmDev<V> A, G g_in, Epi epi) {
	constexpr int NV = Epi::NV;
	__shared__ double red[128];
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	G g = g_in;
	g.init();
	Acc<V, NV> acc;
	acc.init();
	const int segs = (A.nx + kFvmThreads - 1) / kFvmThreads;
	const int G0 = (int)gridDim.x;
	// position of tile blockIdx.x and the step G0 as (segment, j, k)
	int seg = (int)blockIdx.x % segs, line = (int)blockIdx.x / segs;
	int j = line % A.ny, k = line / A.ny;
	const int dseg = G0 % segs, dline = G0 / segs;
	const int dj = dline % A.ny, dk = dline / A.ny;
	while (k < A.nz) {
		const int i = seg * kFvmThreads + (int)threadIdx.x;
		if (i < A.nx) {
			const int r = (k * A.ny + j) * A.nx + i;
			epi.row(r, fvm_cell<V, TF, AV>(A, g, i, j, k, r), acc);
		}
		seg += dseg;
		j += dj;
		k += dk;
		if (seg >= segs) {
			seg -= segs;
			++j;
		}
		if (j >= A.ny) {
			j -= A.ny;
			++k;
		}
	}
	if constexpr (NV > 0) {
		acc.to_part(epi.part, red);
		if (last_block(epi.counter)) {
			double sums[NV];
			sum_partials<NV>(epi.part, gridDim.x, sums, red);
			if (threadIdx.x == 0) {
				epi.finish(sums);
				*epi.counter = 0;
			}
		}
	}
}

// Plane-marching form for FP64 on meshes at least one warp wide.  A CTA covers a
// 32 x 8 tile of (x, y) columns and marches kFvmZ planes up in z; each warp
// is one x row of the tile.  Per thread the cell below, the cell and the cell
// above are kept in registers (one new load per plane), the x neighbours come
// from the neighbouring lanes, and two fluxes are shared instead of computed
// twice: a cell's low x flux is the high x flux of the lane before it, and
// its low z flux the high z flux of the plane before.  A shared flux is the
// product of the same two operands, so v is the same bit for bit as the
// per-cell form.
constexpr int kFvmTileX = 32, kFvmTileY = 8, kFvmZ = 16;

template<class V, bool TF, bool AV, class G, class Epi>
__global__ void __launch_bounds__(kFvmTileX * kFvmTileY)
spmv_fvm3_kernel(FvmDev<V> A, G g_in, Epi epi) {
	constexpr int NV = Epi::NV;
	constexpr unsigned kFull = 0xffffffffu;
	__shared__ double red[128];
	pdl_wait();
	pdl_trigger();
	if (epi.skip())
		return;
	G g = g_in;
	g.init();
	Acc<V, NV> acc;
	acc.init();
	const int nx = A.nx, ny = A.ny, nz = A.nz;
	const int fx = nx + 1, fxy = fx * (ny + 1), plane = nx * ny;
	const int tx = (int)threadIdx.x & 31, ty = (int)threadIdx.x >> 5;
	const int tiles_x = (nx + kFvmTileX - 1) / kFvmTileX, tiles_y = (ny + kFvmTileY - 1) / kFvmTileY;
	const int tiles_xy = tiles_x * tiles_y;
	const int ntile = tiles_xy * ((nz + kFvmZ - 1) / kFvmZ);
	for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
		const int bz = t / tiles_xy, bxy = t - bz * tiles_xy;
		const int by = bxy / tiles_x, bx = bxy - by * tiles_x;
		const int i = bx * kFvmTileX + tx, j = by * kFvmTileY + ty, k0 = bz * kFvmZ;
		const int k1 = min(k0 + kFvmZ, nz);
		// the column is in the mesh; a lane outside it (a partial tile) loads
		// nothing and keeps index 0, taking part only in the shuffles
		const bool in = i < nx && j < ny;
		int r = in ? (k0 * ny + j) * nx + i : 0;
		int ix = in ? ((k0 + 1) * (ny + 1) + (j + 1)) * fx + i : 0;  // x face i (low) of cell (i, j, k)
		V uc = in ? g.at(r) : V(0);
		V ub = (in && k0 > 0) ? g.at(r - plane) : V(0);
		V fz_carry = V(0);
		for (int k = k0; k < k1; ++k) {
			const V ua = (in && k + 1 < nz) ? g.at(r + plane) : V(0);
			const V ud = k > 0 ? ub : fvm_ghost(A, 4, uc);
			const V uu = k + 1 < nz ? ua : fvm_ghost(A, 5, uc);
			// x neighbours: the lanes either side, a load at the warp's
			// edges, the boundary value at the mesh's
			const V w_sh = __shfl_up_sync(kFull, uc, 1);
			const V e_sh = __shfl_down_sync(kFull, uc, 1);
			V ue;
			if (i + 1 >= nx)
				ue = fvm_ghost(A, 1, uc);
			else
				ue = tx < 31 ? e_sh : (in ? g.at(r + 1) : V(0));
			const V fx_hi = in ? mul_rn(fvm_t<V, TF>(A, 0, ix + 1), sub_rn(ue, uc)) : V(0);
			const V fx_sh = __shfl_up_sync(kFull, fx_hi, 1);
			V fx_lo;
			if (tx > 0 && i > 0)
				fx_lo = fx_sh;
			else {
				const V uw = i > 0 ? (tx > 0 ? w_sh : (in ? g.at(r - 1) : V(0))) : fvm_ghost(A, 0, uc);
				fx_lo = in ? mul_rn(fvm_t<V, TF>(A, 0, ix), sub_rn(uc, uw)) : V(0);
			}
			const int iy = ix + 1 - fx;
			const V us = j > 0 ? (in ? g.at(r - nx) : V(0)) : fvm_ghost(A, 2, uc);
			const V un = j + 1 < ny ? (in ? g.at(r + nx) : V(0)) : fvm_ghost(A, 3, uc);
			const V fy_hi = in ? mul_rn(fvm_t<V, TF>(A, 1, iy + fx), sub_rn(un, uc)) : V(0);
			const V fy_lo = in ? mul_rn(fvm_t<V, TF>(A, 1, iy), sub_rn(uc, us)) : V(0);
			const V fz_hi = in ? mul_rn(fvm_t<V, TF>(A, 2, ix + 1), sub_rn(uu, uc)) : V(0);
			const V fz_lo = k > k0 ? fz_carry
			                       : (in ? mul_rn(fvm_t<V, TF>(A, 2, ix + 1 - fxy), sub_rn(uc, ud)) : V(0));
			const V du = add_rn(add_rn(sub_rn(fx_hi, fx_lo), sub_rn(fy_hi, fy_lo)), sub_rn(fz_hi, fz_lo));
			V av;
			if constexpr (AV)
				av = in ? __ldg(A.av + r) : V(0);
			else
				av = A.avc;
			if (in)
				epi.row(r, add_rn(mul_rn(A.neg_beta, du), mul_rn(av, uc)), acc);
			fz_carry = fz_hi;
			ub = uc;
			uc = ua;
			if (in) {
				r += plane;
				ix += fxy;
			}
		}
	}
	if constexpr (NV > 0) {
		acc.to_part(epi.part, red);
		if (last_block(epi.counter)) {
			double sums[NV];
			sum_partials<NV>(epi.part, gridDim.x, sums, red);
			if (threadIdx.x == 0) {
				epi.finish(sums);
				*epi.counter = 0;
			}
		}
	}
}

template<class V, bool TF, bool AV, class G, class Epi>
static inline int launch_spmv_fvm_as(Ctx *ctx, const FvmOp *op, const G &g, const Epi &epi) {
	// FP64 is bound by its pipe, and the marching form does 16 FP64 operations
	// per cell instead of 20; FP32 is bound by load latency, which the
	// per-cell form hides better (0.083 against 0.111 ms at 256^3)
	if (sizeof(V) == 8 && op->nx >= kFvmTileX) {
		const int64_t ntile = (int64_t)((op->nx + kFvmTileX - 1) / kFvmTileX) *
		                      ((op->ny + kFvmTileY - 1) / kFvmTileY) * ((op->nz + kFvmZ - 1) / kFvmZ);
		const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntile, (int64_t)ctx->sms * 8));
		return check_launch_rc(ctx, launch_pdl(ctx->stream, spmv_fvm3_kernel<V, TF, AV, G, Epi>, grid,
		                                       kFvmTileX * kFvmTileY, 0, op->dev<V>(), g, epi),
		                       "spmv (finite-volume stencil, plane marching)");
	}
	const int segs = (op->nx + kFvmThreads - 1) / kFvmThreads;
	const int64_t ntile = (int64_t)segs * op->ny * op->nz;
	const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntile, (int64_t)ctx->sms * 8));
	return check_launch_rc(ctx, launch_pdl(ctx->stream, spmv_fvm_kernel<V, TF, AV, G, Epi>, grid, kFvmThreads, 0,
	                                       op->dev<V>(), g, epi),
	                       "spmv (finite-volume stencil)");
}

template<class V, class G, class Epi>
static inline int launch_spmv_fvm(Ctx *ctx, const FvmOp *op, const G &g, const Epi &epi) {
	const bool tf = op->t64[0] != nullptr, av = op->av64 != nullptr;
	if (tf)
		return av ? launch_spmv_fvm_as<V, true, true>(ctx, op, g, epi)
		          : launch_spmv_fvm_as<V, true, false>(ctx, op, g, epi);
	return av ? launch_spmv_fvm_as<V, false, true>(ctx, op, g, epi)
	          : launch_spmv_fvm_as<V, false, false>(ctx, op, g, epi);
}

}  // namespace fsg
