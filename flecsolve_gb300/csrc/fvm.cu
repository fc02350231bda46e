// Finite-volume physics operators on the device.
//
// Two layers:
//  * the reference's physics operators one for one, on fields with their
//    boundary layer (flecsolve/physics/): the Dirichlet and Neumann boundary
//    operators (boundary/dirichlet.hh:49-63, boundary/neumann.hh:49-74), the
//    constant and average face-coefficient setters
//    (volume_diffusion/coefficient.hh:84-177) and the volume diffusion
//    operator (volume_diffusion/diffusion.hh:109-193, flux, surface sum and
//    volume term fused into one sweep).  Same IEEE operations in the same
//    order, so the fields are identical bit for bit;
//  * the matrix-free operator the solvers apply (spmv_fvm.cuh): boundary
//    operators on all six faces, a face coefficient (fields or a constant)
//    and the diffusion operator, on vectors of the logical cells.  It is an
//    fs_csr handle without stored rows: operator applies, residuals, the
//    Jacobi diagonal and every Krylov solver accept it.
//
// Mesh: the specialization's geometry (physics/specializations/
// fvm_narray.hh:233-289): spacing dx = |hi - lo| / (cells including the
// boundary layers - 1), face area dA = the product of the other two
// spacings and cell volume = the product of all three, both folded from the
// right onto 1.0; the flux factor of a face is dA * (1 / dx).
#include <cmath>
#include <cstdint>

#include "fsgpu_internal.cuh"
#include "spmv_kernel.cuh"

namespace fsg {

namespace {

struct Mesh {
	int64_t n[3];
	double dx[3], dA[3], vol, c[3];
	int64_t C, F, N;  // cell-field, face-field and logical-cell counts
	int64_t cell(int64_t I, int64_t J, int64_t K) const { return (K * (n[1] + 2) + J) * (n[0] + 2) + I; }
};

int mesh_of(const fs_fvm_mesh *m, Mesh &g) {
	if (!m)
		return FS_ERR_INVALID_ARG;
	for (int a = 0; a < 3; ++a) {
		g.n[a] = m->n[a];
		if (g.n[a] < 1 || g.n[a] > (1 << 20))
			return FS_ERR_INVALID_ARG;
		if (!std::isfinite(m->box[a][0]) || !std::isfinite(m->box[a][1]))
			return FS_ERR_INVALID_ARG;
	}
	g.C = (g.n[0] + 2) * (g.n[1] + 2) * (g.n[2] + 2);
	g.F = (g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
	g.N = g.n[0] * g.n[1] * g.n[2];
	if (g.C >= ((int64_t)1 << 31))
		return FS_ERR_INVALID_ARG;
	for (int a = 0; a < 3; ++a)
		g.dx[a] = std::abs(m->box[a][1] - m->box[a][0]) / (double)(uint64_t)(g.n[a] + 2 - 1);
	g.dA[0] = g.dx[1] * (g.dx[2] * 1.0);
	g.dA[1] = g.dx[0] * (g.dx[2] * 1.0);
	g.dA[2] = g.dx[0] * (g.dx[1] * 1.0);
	g.vol = g.dx[0] * (g.dx[1] * (g.dx[2] * 1.0));
	for (int a = 0; a < 3; ++a)
		g.c[a] = g.dA[a] * (1.0 / g.dx[a]);
	return FS_OK;
}

// n as int3 for the kernels
struct Dims {
	int nx, ny, nz;
};
Dims dims(const Mesh &g) { return {(int)g.n[0], (int)g.n[1], (int)g.n[2]}; }

__device__ __forceinline__ int64_t cell_idx(const Dims &d, int I, int J, int K) {
	return ((int64_t)K * (d.ny + 2) + J) * (d.nx + 2) + I;
}
__device__ __forceinline__ int64_t face_idx(const Dims &d, int I, int J, int K) {
	return ((int64_t)K * (d.ny + 1) + J) * (d.nx + 1) + I;
}

// Boundary operator on one face: the boundary cells beyond it (the other two
// axes over their logical cells) get the Dirichlet value, or for a Neumann
// face the neighbouring logical cell's value minus (nd dx) q.
__global__ void k_fvm_boundary(Dims d, int face, int kind, double value, double *__restrict__ u) {
	const int axis = face / 2;
	const bool low = (face & 1) == 0;
	const int na = axis == 0 ? d.ny : d.nx;            // first other axis
	const int nb = axis == 2 ? d.ny : d.nz;            // second other axis
	const int64_t cnt = (int64_t)na * nb;
	for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
		const int p = 1 + (int)(t % na), q = 1 + (int)(t / na);
		const int nax = axis == 0 ? d.nx : axis == 1 ? d.ny : d.nz;
		const int b = low ? 0 : nax + 1, in = low ? 1 : nax;
		int64_t gi, ii;
		if (axis == 0) {
			gi = cell_idx(d, b, p, q);
			ii = cell_idx(d, in, p, q);
		}
		else if (axis == 1) {
			gi = cell_idx(d, p, b, q);
			ii = cell_idx(d, p, in, q);
		}
		else {
			gi = cell_idx(d, p, q, b);
			ii = cell_idx(d, p, q, in);
		}
		u[gi] = kind == kFvmBcDirichlet ? value : __dsub_rn(u[ii], value);
	}
}

// Face coefficients of one axis: faces 0..n along it, the other two axes
// over their logical cells; the constant, or the average of the two cells
// either side of the face.
template<bool AVERAGE>
__global__ void k_fvm_coef(Dims d, int axis, double value, const double *__restrict__ u, double *__restrict__ b) {
	// extents and first index of the range per axis, x fastest
	const int ex = d.nx + (axis == 0), ey = d.ny + (axis == 1), ez = d.nz + (axis == 2);
	const int ox = axis != 0, oy = axis != 1, oz = axis != 2;
	const int64_t cnt = (int64_t)ex * ey * ez;
	const int64_t up = axis == 0 ? 1 : axis == 1 ? (int64_t)(d.nx + 2) : (int64_t)(d.nx + 2) * (d.ny + 2);
	for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
		const int I = ox + (int)(t % ex), J = oy + (int)((t / ex) % ey), K = oz + (int)(t / ((int64_t)ex * ey));
		double v = value;
		if constexpr (AVERAGE) {
			const int64_t lo = cell_idx(d, I, J, K);
			v = __dmul_rn(0.5, __dadd_rn(u[lo + up], u[lo]));
		}
		b[face_idx(d, I, J, K)] = v;
	}
}

// Volume diffusion on the logical cells of fields with their boundary layer
// (diffusion.hh:109-193): per face flux (b (dA * (1/dx))) (u_hi - u_lo), the
// cell's surface sum (x, then y, then z differences of its two faces) and
// v = (-beta) du + ((alpha vol) a) u.
__global__ void k_fvm_diffusion(Dims d, double c0, double c1, double c2, double neg_beta, double alpha_vol,
                                const double *__restrict__ a, const double *__restrict__ bx,
                                const double *__restrict__ by, const double *__restrict__ bz,
                                const double *__restrict__ u, double *__restrict__ v) {
	const int64_t cnt = (int64_t)d.nx * d.ny * d.nz;
	const int64_t sy = d.nx + 2, sz = (int64_t)(d.nx + 2) * (d.ny + 2);
	const int64_t fy = d.nx + 1, fz = (int64_t)(d.nx + 1) * (d.ny + 1);
	for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
		const int I = 1 + (int)(t % d.nx), J = 1 + (int)((t / d.nx) % d.ny),
		          K = 1 + (int)(t / ((int64_t)d.nx * d.ny));
		const int64_t c = cell_idx(d, I, J, K), f = face_idx(d, I, J, K);
		const double uc = u[c];
		const double fx_hi = __dmul_rn(__dmul_rn(bx[f], c0), __dsub_rn(u[c + 1], uc));
		const double fx_lo = __dmul_rn(__dmul_rn(bx[f - 1], c0), __dsub_rn(uc, u[c - 1]));
		const double fy_hi = __dmul_rn(__dmul_rn(by[f], c1), __dsub_rn(u[c + sy], uc));
		const double fy_lo = __dmul_rn(__dmul_rn(by[f - fy], c1), __dsub_rn(uc, u[c - sy]));
		const double fz_hi = __dmul_rn(__dmul_rn(bz[f], c2), __dsub_rn(u[c + sz], uc));
		const double fz_lo = __dmul_rn(__dmul_rn(bz[f - fz], c2), __dsub_rn(uc, u[c - sz]));
		const double du = __dadd_rn(__dadd_rn(__dsub_rn(fx_hi, fx_lo), __dsub_rn(fy_hi, fy_lo)),
		                            __dsub_rn(fz_hi, fz_lo));
		v[c] = __dadd_rn(__dmul_rn(neg_beta, du), __dmul_rn(__dmul_rn(alpha_vol, a[c]), uc));
	}
}

// logical cells <-> fields with a boundary layer
template<bool TO_FIELD>
__global__ void k_fvm_pack(Dims d, double *__restrict__ field, double *__restrict__ x) {
	const int64_t cnt = (int64_t)d.nx * d.ny * d.nz;
	for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
		const int I = 1 + (int)(t % d.nx), J = 1 + (int)((t / d.nx) % d.ny),
		          K = 1 + (int)(t / ((int64_t)d.nx * d.ny));
		if constexpr (TO_FIELD)
			field[cell_idx(d, I, J, K)] = x[t];
		else
			x[t] = field[cell_idx(d, I, J, K)];
	}
}

// transmissibilities t = b c of one axis (FP64 and FP32)
__global__ void k_fvm_trans(int64_t n, double c, const double *__restrict__ b, double *__restrict__ t64,
                            float *__restrict__ t32) {
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double t = __dmul_rn(b[i], c);
		t64[i] = t;
		t32[i] = (float)t;
	}
}

// (alpha vol) a per logical cell
__global__ void k_fvm_av(Dims d, double alpha_vol, const double *__restrict__ a, double *__restrict__ av64,
                         float *__restrict__ av32) {
	const int64_t cnt = (int64_t)d.nx * d.ny * d.nz;
	for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
		const int I = 1 + (int)(t % d.nx), J = 1 + (int)((t / d.nx) % d.ny),
		          K = 1 + (int)(t / ((int64_t)d.nx * d.ny));
		const double v = __dmul_rn(alpha_vol, a[cell_idx(d, I, J, K)]);
		av64[t] = v;
		av32[t] = (float)v;
	}
}

// Jacobi diagonal of the matrix-free operator: dv_r / du_r = beta S + (alpha
// vol) a_r, S the sum of the cell's six transmissibilities (x pair, y pair,
// z pair), a Neumann face contributing none (its flux does not depend on u)
__global__ void k_fvm_dinv(FvmDev<double> A, double beta, double *__restrict__ dinv, float *__restrict__ dinv32) {
	const int64_t cnt = (int64_t)A.nx * A.ny * A.nz;
	const int64_t fx = (int64_t)A.nx + 1, fxy = fx * (A.ny + 1);
	for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += (int64_t)gridDim.x * blockDim.x) {
		const int i = (int)(t % A.nx), j = (int)((t / A.nx) % A.ny), k = (int)(t / ((int64_t)A.nx * A.ny));
		const int64_t ix = ((int64_t)(k + 1) * (A.ny + 1) + (j + 1)) * fx + i;
		const int64_t iy = ((int64_t)(k + 1) * (A.ny + 1) + j) * fx + (i + 1);
		const int64_t iz = ((int64_t)k * (A.ny + 1) + (j + 1)) * fx + (i + 1);
		auto tf = [&](int face, bool boundary, int axis, int64_t idx) {
			return boundary && A.ghost_kind[face] == kFvmBcNeumann ? 0.0 : (A.t[axis] ? A.t[axis][idx] : A.tc[axis]);
		};
		const double sx = __dadd_rn(tf(0, i == 0, 0, ix), tf(1, i + 1 == A.nx, 0, ix + 1));
		const double sy = __dadd_rn(tf(2, j == 0, 1, iy), tf(3, j + 1 == A.ny, 1, iy + fx));
		const double sz = __dadd_rn(tf(4, k == 0, 2, iz), tf(5, k + 1 == A.nz, 2, iz + fxy));
		const double av = A.av ? A.av[t] : A.avc;
		const double diag = __dadd_rn(__dmul_rn(beta, __dadd_rn(__dadd_rn(sx, sy), sz)), av);
		const double di = diag != 0.0 ? 1.0 / diag : 0.0;
		dinv[t] = di;
		dinv32[t] = (float)di;
	}
}

int grid_of(Ctx *ctx, int64_t n) { return grid_for(ctx, std::max<int64_t>(n, 1), 256, 4); }

bool field_ok(const Vec *v, int64_t n) { return ok_vec(v) && v->n == n && v->dtype == FS_F64; }

}  // namespace

}  // namespace fsg

using namespace fsg;

extern "C" {

FS_API int fs_fvm_geometry(const fs_fvm_mesh *m, double dx[3], double dA[3], double *volume) {
	Mesh g;
	FS_TRY(mesh_of(m, g));
	for (int a = 0; a < 3; ++a) {
		if (dx)
			dx[a] = g.dx[a];
		if (dA)
			dA[a] = g.dA[a];
	}
	if (volume)
		*volume = g.vol;
	return FS_OK;
}

FS_API int fs_fvm_boundary(fs_ctx h, const fs_fvm_mesh *m, int face, int kind, double value, fs_vec uh) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Vec *u = reinterpret_cast<Vec *>(uh);
	if (!ok_ctx(ctx) || !ok_vec(u))
		return FS_ERR_BAD_HANDLE;
	Mesh g;
	if (mesh_of(m, g) != FS_OK || face < 0 || face > 5 || (kind != FS_BC_DIRICHLET && kind != FS_BC_NEUMANN))
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_boundary: bad mesh, face or kind");
	if (!field_ok(u, g.C))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_boundary: u is not an FP64 cell field of the mesh");
	// Neumann: the shift (nd dx) q, nd = +1 on a low face, -1 on a high one
	const int axis = face / 2;
	const double nd = (face & 1) == 0 ? 1.0 : -1.0;
	const double v = kind == FS_BC_DIRICHLET ? value : (nd * g.dx[axis]) * value;
	const int64_t cnt = (axis == 0 ? g.n[1] * g.n[2] : axis == 1 ? g.n[0] * g.n[2] : g.n[0] * g.n[1]);
	k_fvm_boundary<<<grid_of(ctx, cnt), 256, 0, ctx->stream>>>(dims(g), face, kind, v, (double *)u->d);
	return check_launch(ctx, "fvm boundary");
}

static int coef(fs_ctx h, const fs_fvm_mesh *m, bool average, double value, fs_vec uh, fs_vec bxh, fs_vec byh,
                fs_vec bzh) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Vec *u = reinterpret_cast<Vec *>(uh);
	Vec *b[3] = {reinterpret_cast<Vec *>(bxh), reinterpret_cast<Vec *>(byh), reinterpret_cast<Vec *>(bzh)};
	if (!ok_ctx(ctx) || !ok_vec(b[0]) || !ok_vec(b[1]) || !ok_vec(b[2]) || (average && !ok_vec(u)))
		return FS_ERR_BAD_HANDLE;
	Mesh g;
	if (mesh_of(m, g) != FS_OK)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_coef: bad mesh");
	for (auto *bb : b)
		if (!field_ok(bb, g.F))
			return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_coef: a face field does not fit the mesh");
	if (average && !field_ok(u, g.C))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_coef_average: u is not a cell field of the mesh");
	for (int a = 0; a < 3; ++a) {
		const int64_t cnt = (g.n[a] + 1) * (g.N / g.n[a]);
		if (average)
			k_fvm_coef<true><<<grid_of(ctx, cnt), 256, 0, ctx->stream>>>(dims(g), a, 0.0, (const double *)u->d,
			                                                             (double *)b[a]->d);
		else
			k_fvm_coef<false><<<grid_of(ctx, cnt), 256, 0, ctx->stream>>>(dims(g), a, value, nullptr,
			                                                              (double *)b[a]->d);
		FS_TRY(check_launch(ctx, "fvm coefficient"));
	}
	return FS_OK;
}

FS_API int fs_fvm_coef_constant(fs_ctx h, const fs_fvm_mesh *m, double value, fs_vec bx, fs_vec by, fs_vec bz) {
	return coef(h, m, false, value, nullptr, bx, by, bz);
}

FS_API int fs_fvm_coef_average(fs_ctx h, const fs_fvm_mesh *m, fs_vec u, fs_vec bx, fs_vec by, fs_vec bz) {
	return coef(h, m, true, 0.0, u, bx, by, bz);
}

FS_API int fs_fvm_diffusion(fs_ctx h, const fs_fvm_mesh *m, double beta, double alpha, fs_vec ah, fs_vec bxh,
                            fs_vec byh, fs_vec bzh, fs_vec uh, fs_vec vh) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Vec *a = reinterpret_cast<Vec *>(ah), *u = reinterpret_cast<Vec *>(uh), *v = reinterpret_cast<Vec *>(vh);
	Vec *b[3] = {reinterpret_cast<Vec *>(bxh), reinterpret_cast<Vec *>(byh), reinterpret_cast<Vec *>(bzh)};
	if (!ok_ctx(ctx) || !ok_vec(a) || !ok_vec(u) || !ok_vec(v) || !ok_vec(b[0]) || !ok_vec(b[1]) || !ok_vec(b[2]))
		return FS_ERR_BAD_HANDLE;
	Mesh g;
	if (mesh_of(m, g) != FS_OK)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_diffusion: bad mesh");
	if (!field_ok(a, g.C) || !field_ok(u, g.C) || !field_ok(v, g.C) || !field_ok(b[0], g.F) ||
	    !field_ok(b[1], g.F) || !field_ok(b[2], g.F))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_diffusion: a field does not fit the mesh");
	if (u == v)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_diffusion: u and v must differ");
	k_fvm_diffusion<<<grid_of(ctx, g.N), 256, 0, ctx->stream>>>(
		dims(g), g.c[0], g.c[1], g.c[2], -beta, alpha * g.vol, (const double *)a->d, (const double *)b[0]->d,
		(const double *)b[1]->d, (const double *)b[2]->d, (const double *)u->d, (double *)v->d);
	return check_launch(ctx, "fvm diffusion");
}

static int pack(fs_ctx h, const fs_fvm_mesh *m, fs_vec fh, fs_vec xh, bool to_field) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	Vec *f = reinterpret_cast<Vec *>(fh), *x = reinterpret_cast<Vec *>(xh);
	if (!ok_ctx(ctx) || !ok_vec(f) || !ok_vec(x))
		return FS_ERR_BAD_HANDLE;
	Mesh g;
	if (mesh_of(m, g) != FS_OK)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_pack: bad mesh");
	if (!field_ok(f, g.C) || !field_ok(x, g.N))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_pack: sizes do not fit the mesh");
	if (to_field)
		k_fvm_pack<true><<<grid_of(ctx, g.N), 256, 0, ctx->stream>>>(dims(g), (double *)f->d, (double *)x->d);
	else
		k_fvm_pack<false><<<grid_of(ctx, g.N), 256, 0, ctx->stream>>>(dims(g), (double *)f->d, (double *)x->d);
	return check_launch(ctx, "fvm pack");
}

FS_API int fs_fvm_pack(fs_ctx h, const fs_fvm_mesh *m, fs_vec field, fs_vec x) {
	return pack(h, m, field, x, false);
}

FS_API int fs_fvm_unpack(fs_ctx h, const fs_fvm_mesh *m, fs_vec x, fs_vec field) {
	return pack(h, m, field, x, true);
}

FS_API int fs_fvm_operator_create(fs_ctx h, const fs_fvm_operator_settings *s, fs_vec ah, fs_vec bxh, fs_vec byh,
                                  fs_vec bzh, fs_csr *out) {
	Ctx *ctx = reinterpret_cast<Ctx *>(h);
	if (!ok_ctx(ctx) || !s || !out)
		return FS_ERR_BAD_HANDLE;
	*out = nullptr;
	Vec *a = reinterpret_cast<Vec *>(ah);
	Vec *b[3] = {reinterpret_cast<Vec *>(bxh), reinterpret_cast<Vec *>(byh), reinterpret_cast<Vec *>(bzh)};
	Mesh g;
	if (mesh_of(&s->mesh, g) != FS_OK)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_operator_create: bad mesh");
	if (g.N >= ((int64_t)1 << 31) - 64)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_operator_create: too many cells");
	for (int f = 0; f < 6; ++f)
		if (s->bc_kind[f] != FS_BC_DIRICHLET && s->bc_kind[f] != FS_BC_NEUMANN)
			return set_err(ctx, FS_ERR_INVALID_ARG,
			               "fs_fvm_operator_create: every face needs a Dirichlet or Neumann boundary");
	const int nfaces = (b[0] != nullptr) + (b[1] != nullptr) + (b[2] != nullptr);
	if (nfaces != 0 && nfaces != 3)
		return set_err(ctx, FS_ERR_INVALID_ARG, "fs_fvm_operator_create: give all three face fields or none");
	for (int k = 0; k < nfaces; ++k)
		if (!field_ok(b[k], g.F))
			return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_operator_create: a face field does not fit the mesh");
	if (a && !field_ok(a, g.C))
		return set_err(ctx, FS_ERR_SIZE_MISMATCH, "fs_fvm_operator_create: a is not a cell field of the mesh");

	FvmOp *op = new FvmOp();
	Csr *A = new Csr();
	A->ctx = ctx;
	A->nrows = A->ncols = g.N;
	A->nnz = g.N + 2 * ((g.n[0] - 1) * g.n[1] * g.n[2] + g.n[0] * (g.n[1] - 1) * g.n[2] +
	                    g.n[0] * g.n[1] * (g.n[2] - 1));
	A->fvm = op;
	auto fail = [&](int st) {
		fs_csr_destroy(reinterpret_cast<fs_csr>(A));
		return st;
	};
	op->nx = (int)g.n[0];
	op->ny = (int)g.n[1];
	op->nz = (int)g.n[2];
	op->beta = s->beta;
	op->alpha = s->alpha;
	for (int k = 0; k < 3; ++k) {
		op->dx[k] = g.dx[k];
		op->dA[k] = g.dA[k];
		op->c[k] = g.c[k];
	}
	op->vol = g.vol;
	for (int f = 0; f < 6; ++f) {
		op->bc_kind[f] = s->bc_kind[f];
		op->bc_value[f] = s->bc_value[f];
		const double nd = (f & 1) == 0 ? 1.0 : -1.0;
		op->ghost[f] = s->bc_kind[f] == FS_BC_DIRICHLET ? s->bc_value[f] : (nd * g.dx[f / 2]) * s->bc_value[f];
		if (s->bc_value[f] != 0.0)
			op->affine = true;
	}
	const double alpha_vol = s->alpha * g.vol;
	if (nfaces == 0)
		for (int k = 0; k < 3; ++k)
			op->tc[k] = s->b_value * g.c[k];
	else
		for (int k = 0; k < 3; ++k) {
			if (cudaMalloc(&op->t64[k], (size_t)g.F * sizeof(double)) != cudaSuccess ||
			    cudaMalloc(&op->t32[k], (size_t)g.F * sizeof(float)) != cudaSuccess)
				return fail(set_err(ctx, FS_ERR_OUT_OF_MEMORY, "fs_fvm_operator_create: out of device memory"));
			k_fvm_trans<<<grid_of(ctx, g.F), 256, 0, ctx->stream>>>(g.F, g.c[k], (const double *)b[k]->d,
			                                                      op->t64[k], op->t32[k]);
			if (int st = check_launch(ctx, "fvm transmissibilities"))
				return fail(st);
		}
	if (a) {
		if (cudaMalloc(&op->av64, (size_t)g.N * sizeof(double)) != cudaSuccess ||
		    cudaMalloc(&op->av32, (size_t)g.N * sizeof(float)) != cudaSuccess)
			return fail(set_err(ctx, FS_ERR_OUT_OF_MEMORY, "fs_fvm_operator_create: out of device memory"));
		k_fvm_av<<<grid_of(ctx, g.N), 256, 0, ctx->stream>>>(dims(g), alpha_vol, (const double *)a->d, op->av64,
		                                                   op->av32);
		if (int st = check_launch(ctx, "fvm cell coefficient"))
			return fail(st);
	}
	else
		op->avc = alpha_vol * s->a_value;
	const size_t padded = (size_t)((g.N + 31) / 32 * 32 + 32);
	if (cudaMalloc(&A->dinv, padded * sizeof(double)) != cudaSuccess ||
	    cudaMalloc(&A->dinv32, padded * sizeof(float)) != cudaSuccess)
		return fail(set_err(ctx, FS_ERR_OUT_OF_MEMORY, "fs_fvm_operator_create: out of device memory"));
	cudaMemsetAsync(A->dinv, 0, padded * sizeof(double), ctx->stream);
	cudaMemsetAsync(A->dinv32, 0, padded * sizeof(float), ctx->stream);
	k_fvm_dinv<<<grid_of(ctx, g.N), 256, 0, ctx->stream>>>(op->dev<double>(), s->beta, A->dinv, A->dinv32);
	if (int st = check_launch(ctx, "fvm diagonal"))
		return fail(st);
	A->dinv_valid = true;
	A->val32_valid = true;
	*out = reinterpret_cast<fs_csr>(A);
	return FS_OK;
}

FS_API int fs_fvm_operator_info(fs_csr h, int *affine, int64_t dims_out[3]) {
	Csr *A = reinterpret_cast<Csr *>(h);
	if (!ok_csr(A))
		return FS_ERR_BAD_HANDLE;
	if (!A->fvm)
		return set_err(A->ctx, FS_ERR_INVALID_ARG, "fs_fvm_operator_info: not a finite-volume operator");
	if (affine)
		*affine = A->fvm->affine ? 1 : 0;
	if (dims_out) {
		dims_out[0] = A->fvm->nx;
		dims_out[1] = A->fvm->ny;
		dims_out[2] = A->fvm->nz;
	}
	return FS_OK;
}

}  // extern "C"

namespace fsg {

void destroy_fvm(FvmOp *op) {
	if (!op)
		return;
	for (int k = 0; k < 3; ++k) {
		if (op->t64[k])
			cudaFree(op->t64[k]);
		if (op->t32[k])
			cudaFree(op->t32[k]);
	}
	if (op->av64)
		cudaFree(op->av64);
	if (op->av32)
		cudaFree(op->av32);
	delete op;
}

}  // namespace fsg
