// Bound Krylov solver object shared by krylov.cu and gmres.cu.
//
// One fs_solver is the device counterpart of an op::core<op::cg<params>>
// (flecsolve/solvers/krylov_parameters.hh:94-126): settings, work vectors,
// operator, preconditioner and diagnostic, plus the device-resident scalar
// state of the running solve and the CUDA graphs of its iteration body.
#pragma once

#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "spmv_kernel.cuh"

namespace fsg {

// flags
constexpr int KF_NEG_CURVATURE = 1;   // CG: p'Ap <= 0 (cg.hh:101-104 logs it)
constexpr int KF_ALPHA_ZERO = 2;      // BiCGSTAB: r~'v == 0 (bicgstab.hh:129)
constexpr int KF_RESTART = 4;         // BiCGSTAB: restart requested (bicgstab.hh:103)
constexpr int KF_EARLY = 8;           // BiCGSTAB: ||s|| < rtol early exit (bicgstab.hh:136)
constexpr int KF_NONFINITE = 16;      // a reduction produced NaN/Inf
constexpr int KF_RELIABLE = 32;       // mixed CG: residual replacement due

// Device-resident scalars of one solve.  Written only by the last block of a
// reduction kernel (thread 0); read by every kernel that follows.
struct KState {
	double bnorm, tol, rtol;          // rhs norm (after the zero fix-up), terminate_tol
	double rhs_norm;                  // info.rhs_norm as the reference reports it
	double sol0, res0;                // initial solution / residual norms
	double res;                       // current residual norm
	double rho, rho_old, alpha, beta, omega, pAp;
	double r_tilde_norm, s_norm, t_sq, t_s;
	double aux[4];
	double alpha_x;                   // reliable CG: step of the pending xs += alpha p
	int iter;                         // iterations completed (loop counter)
	int done;                         // nonzero: stop
	int status;                       // fs_stop_reason
	int info_iters;                   // info.iters as the reference sets it
	int flags;
	int maxiter;
	int restarts;
	int hist_cap;
	int nhist;                        // history entries written
	int pad_;
};

// GMRES least-squares state (gmres.cu): Hessenberg (column-major, ld = m+1),
// rotations, right-hand side, back-solve result, the projections of the step
constexpr int kGmMaxDim = 100;  // gmres.hh:31 krylov_dim_bound
constexpr int kGmDelayedCols = 32;  // basis columns the delayed CGS2 takes (m <= 30)
constexpr int kPartPerBlock = 32;  // partial sums per CTA a solver kernel may write
struct GmState {
	double H[(kGmMaxDim + 1) * (kGmMaxDim + 1)];
	double cs[kGmMaxDim + 1], sn[kGmMaxDim + 1], dw[kGmMaxDim + 1], dy[kGmMaxDim + 1];
	double h1[kGmMaxDim + 1], h2[kGmMaxDim + 1];
	// delayed CGS2: the Hessenberg columns before the rotations (column k
	// tentative until step k + 1 adds its reorthogonalisation coefficients)
	// and the current step's tau and r
	double Hr[kGmDelayedCols * kGmDelayedCols];
	double dg_tau, dg_r;
	double vnorm;  // H(k+1,k) before the rotation
	int k;         // current Krylov dimension
	int ld;        // Hessenberg leading dimension (min(m, maxiter) + 1)
	int m;         // max_krylov_dim
	int pad_;
};

struct Solver;

struct Precond {
	int kind = FS_PRECOND_NONE;
	Vec *diag = nullptr;
	Csr *op = nullptr;
	Solver *solver = nullptr;   // FS_PRECOND_SOLVER
};

struct GraphKey {
	const void *b, *x;
	int k;
	int fmt = 0;  // SpMV formats in use at capture (set by graph_run)
	bool operator<(const GraphKey &o) const {
		return std::tie(b, x, k, fmt) < std::tie(o.b, o.x, o.k, o.fmt);
	}
};

struct Solver {
	int magic = kMagicSlv;
	Ctx *ctx = nullptr;
	int method = FS_CG;
	fs_krylov_settings set{};
	Csr *A = nullptr;
	Precond P;
	bool pc_diagonal = false;  // an FS_PRECOND_CSR with only diagonal entries
	fs_diag_fn diag = nullptr;
	void *diag_user = nullptr;

	int64_t n = 0;
	// work storage (FP64 and FP32 blocks, allocated on first apply)
	std::vector<void *> bufs;
	double *w64[12] = {};
	float *w32[12] = {};
	double *basis = nullptr;          // GMRES: (m + 1) x n, column j contiguous
	size_t basis_bytes = 0;
	// tensor maps of the basis for the staged CGS2 passes (four CUtensorMap)
	// and what they were encoded for (null base: none)
	alignas(64) unsigned char gm_map[4 * 128];
	const void *gm_map_base = nullptr;
	int gm_map_key[3] = {0, 0, 0};    // element size, columns, n (low 31 bits)
	bool gm_delayed = false;          // this solve orthogonalises with the delayed CGS2
	double *hdev = nullptr;           // GMRES: dot results scratch
	KState *st = nullptr;             // device
	KState *hst = nullptr;            // pinned mirror
	KState *st_in = nullptr;          // device state of an inner solve
	double *hist = nullptr;           // device, residual norm per iteration
	int hist_cap = 0;
	double *part = nullptr;           // reduction partials
	unsigned *counter = nullptr;
	// captured graphs, keyed by the operator they were captured with and the
	// vectors / body they run; at most kMaxGraphs are kept (least recently
	// launched evicted first)
	struct GraphEntry {
		cudaGraphExec_t exec;
		int nodes;
		uint64_t last_use;
	};
	static constexpr size_t kMaxGraphs = 48;
	std::map<std::pair<const Csr *, GraphKey>, GraphEntry> graphs;
	uint64_t graph_tick = 0;
	Csr *AT = nullptr;                // transpose view for the adjoint solve
	std::vector<double> hhist;        // host copy of the last history
	int64_t hhist_count = 0;
	int mixed_outer = 0, mixed_inner = 0;
	int graph_nodes_launched = 0;
	// work vectors of the host-stepped loops (generic.cu), as vector handles
	// the caller's operator callbacks receive
	std::vector<std::unique_ptr<Vec>> gwork;

	const double *dinv64() const;
	const float *dinv32() const;
};

inline bool ok_slv(const Solver *s) { return s && s->magic == kMagicSlv && ok_ctx(s->ctx); }

// largest grid of the elementwise/reduction kernels of a solver
inline int red_grid(Ctx *ctx, int64_t n) { return grid_for(ctx, n, 256, 8); }

// shared helpers (krylov.cu)
int solver_alloc(Solver *s);
int graph_run(Solver *s, const GraphKey &key, int (*body)(Solver *, void *), void *arg);
int read_state(Solver *s);
int solver_norms(Solver *s, Vec *b, Vec *x, bool with_x, int gmres_rule);
int solver_hist(Solver *s, int cap);
int ensure_val32(Csr *A);
int ensure_dinv(Csr *A);

// host-stepped loops for operators and preconditioners the fused device
// loops do not take (generic.cu)
bool needs_generic(const Solver *s);
int generic_apply(Solver *s, Vec *b, Vec *x, fs_solve_info *info);

}  // namespace fsg
