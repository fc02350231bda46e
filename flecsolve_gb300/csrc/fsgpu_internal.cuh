// Internal declarations shared by the translation units of libfsgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "fsgpu.h"

namespace fsg {

constexpr int kMagicCtx = 0x46534358;  // 'FSCX'
constexpr int kMagicVec = 0x46535658;  // 'FSVX'
constexpr int kMagicCsr = 0x46534D58;  // 'FSMX'
constexpr int kMagicSlv = 0x46535358;  // 'FSSX'

// Reduction scratch: one slot of partials per concurrent reduction.
constexpr int kRedThreads = 256;
constexpr int kMaxRedBlocks = 4096;

struct Ctx {
	int magic = kMagicCtx;
	int device = 0;
	int sms = 0;
	cudaStream_t stream = nullptr;
	std::string err;
	int64_t launches = 0;
	// scratch for generic reductions: partials + result + counter
	double *red_part = nullptr;     // kMaxRedBlocks * 4 doubles
	double *red_out = nullptr;      // 8 doubles (device)
	unsigned *red_count = nullptr;  // completion counters (device)
	double *host_out = nullptr;     // pinned
	cudaEvent_t ev[16] = {};        // timing events (fs_ctx_event_*)
	// device error word (bounded waits that ran out); inside red_count
	unsigned *dev_err = nullptr;
};

// reads and clears the device error word (synchronises the stream)
int check_device_error(Ctx *ctx);

struct Vec {
	int magic = kMagicVec;
	Ctx *ctx = nullptr;
	int64_t n = 0;
	int dtype = FS_F64;
	void *d = nullptr;
	bool owns = true;
	size_t bytes() const { return (size_t)n * (dtype == FS_F64 ? 8 : 4); }
};

// Row blocks for the staged CSR SpMV: block b covers rows
// [blk[b], blk[b+1]); a block holds at most kBlkRows rows and kBlkNnz
// nonzeros unless it is a single row longer than kBlkNnz ("long row").
constexpr int kBlkRows = 256;
constexpr int kBlkNnz = 1792;
// row patterns: rows of at most kPatW nonzeros, at most kMaxPat distinct
// sequences of column offsets c - r per matrix
constexpr int kPatW = 8;
constexpr int kMaxPat = 256;

// index formats of the SpMV (fs_csr_index_coding)
constexpr int kCodingColIds = 0;
constexpr int kCodingPatterns = 1;
constexpr int kCodingSym = 2;   // row patterns + symmetric storage (diagonal, upper diagonals)
constexpr int kCodingGrid = 3;  // symmetric storage of a grid stencil: rows addressed by (i, j, k)
constexpr int kCodingGridGen = 4;  // a grid stencil with asymmetric values: diagonal, upper and lower diagonals
constexpr int kMaxSym = 4;      // positive column offsets of the symmetric storage

struct FvmOp;
void destroy_fvm(FvmOp *op);
struct Csr;
void destroy_batch_plans(const Csr *A);

struct Csr {
	int magic = kMagicCsr;
	Ctx *ctx = nullptr;
	int64_t nrows = 0, ncols = 0, nnz = 0;
	int *rowptr = nullptr;     // nrows + 1 (int32 offsets; nnz < 2^31)
	int *col = nullptr;        // nnz (padded to a multiple of 16)
	double *val = nullptr;     // nnz (padded)
	float *val32 = nullptr;    // float copy, built on first use
	bool val32_valid = false;
	unsigned values_gen = 0;   // advanced whenever the values change
	int *blk = nullptr;        // row blocks, nblk + 1
	int4 *blkinfo = nullptr;   // per block {r0, r1, rowptr[r0], rowptr[r1]}
	int nblk = 0;
	// row patterns (null when some row is longer than kPatW or the matrix
	// has more than kMaxPat offset sequences): pattern id per row, kPatW
	// offsets c - r per pattern
	unsigned char *pid = nullptr;
	int *ptab = nullptr;
	int npat = 0;
	unsigned char *plen = nullptr;  // nonzeros per pattern
	short *pwb = nullptr;           // per row block, per 32-row warp: first nonzero - k0
	int coding = kCodingGrid;       // requested format; the next one down when absent
	// symmetric storage (square row-pattern matrices whose patterns pair every
	// offset -d with +d, at most kMaxSym of them): per pattern entry a slot
	// code (0 diagonal, k + 1 upper offset k, -(k + 1) lower offset k), per
	// pattern the entry of each upper offset, the offsets; when the values are
	// symmetric bit for bit, the diagonal and upper diagonals (FP64, FP32),
	// (nsym + 1) x sym_ld each, rebuilt in place when the values change
	signed char *pslot = nullptr;   // npat x kPatW
	signed char *pinv = nullptr;    // npat x kMaxSym (-1: absent)
	int *sofs = nullptr;            // nsym
	int2 *stab = nullptr;           // npat x kPatW: {value offset, column offset} from r
	int nsym = 0;
	int64_t sym_ld = 0;
	// grid stencil (0 when the matrix is none): the symmetric storage's
	// offsets are 1, nx, nx ny (as many as nsym) and row r = i + nx (j + ny k)
	// holds exactly its neighbours inside the nx x ny x nz grid
	int grid_nx = 0, grid_ny = 0, grid_nz = 0;
	double *sym64 = nullptr;
	float *sym32 = nullptr;
	unsigned *sym_flag = nullptr;   // device: set by the build when a pair differs
	bool sym64_valid = false, sym32_valid = false;
	// general grid storage (a grid stencil whose values are not symmetric):
	// the diagonal, the nsym upper diagonals a(r, r + d) and the nsym lower
	// diagonals a(r, r - d), each at row r, (2 nsym + 1) x sym_ld
	double *gen64 = nullptr;
	float *gen32 = nullptr;
	bool gen64_valid = false, gen32_valid = false;
	int sym_state = -1;             // -1 not checked since the values changed, 0 no, 1 yes
	// FMA-mode column-id SpMV kernel per value type (0 FP64, 1 FP32): 0 row
	// blocks, L = 4..32 lanes per row of the vector kernel, 1 the vector
	// kernel with rows binned by length, -1 not tuned yet
	int vec_lanes[2] = {-1, -1};
	// a transposed view (CSC arrays of another CSR, no host offsets): its
	// column-id schedule follows the mean row length, untimed
	bool view = false;
	// the binned schedule (built on first use): row ids grouped by length
	// class, one warp task {first slot, lanes | rows << 8} per 32 / lanes rows
	int *bin_rows = nullptr;
	int2 *bin_task = nullptr;
	int bin_ntask = 0;
	double *dinv = nullptr;    // 1 / a_ii, built on first use
	float *dinv32 = nullptr;
	bool dinv_valid = false;
	// CSC view (transpose) for A^T x
	int *t_colptr = nullptr;   // ncols + 1
	int *t_row = nullptr;      // nnz
	int *t_perm = nullptr;     // nnz: CSC slot -> CSR slot
	double *t_val = nullptr;   // nnz
	int *t_blk = nullptr;
	int4 *t_blkinfo = nullptr;
	int t_nblk = 0;
	bool t_valid = false;
	bool t_vals_valid = false;
	std::vector<int> h_rowptr; // host copy of offsets (parcsr splitting)
	// matrix-free finite-volume operator (no rows, columns or values stored;
	// only the operator applies and the Jacobi diagonal are available)
	FvmOp *fvm = nullptr;
	// caller-defined operator (fs_shell_create): y = shell_fn(shell_user, x,
	// y); nothing stored
	fs_op_fn shell_fn = nullptr;
	void *shell_user = nullptr;
};

// an operator that stores no rows (matrix-free finite-volume or shell)
inline bool stores_no_rows(const Csr *A) { return A->fvm || A->shell_fn; }

// index format an SpMV on A uses (the requested one, or the next one the
// matrix supports)
inline int active_coding(const Csr *A, bool f32 = false) {
	if (!A->pid || A->coding == kCodingColIds)
		return kCodingColIds;
	if (A->coding >= kCodingSym && (f32 ? A->sym32_valid : A->sym64_valid))
		return A->coding == kCodingGrid && A->grid_nx % 4 == 0 && A->grid_nx > 0 ? kCodingGrid
		                                                                         : kCodingSym;
	if (A->coding == kCodingGrid && A->grid_nx % 4 == 0 && A->grid_nx > 0 &&
	    (f32 ? A->gen32_valid : A->gen64_valid))
		return kCodingGridGen;
	return kCodingPatterns;
}

// derived data of A's values (float copy, Jacobi diagonal, CSC values,
// symmetric storage) is stale: rebuilt on next use
void invalidate_values(Csr *A);
// FP32 values and the Jacobi diagonal, built on first use (spmv.cu)
int ensure_val32(Csr *A);
// lanes per row of the FMA-mode column-id SpMV for A's values of one type (0:
// the row-block kernel); tunes A on first use outside a graph capture
int spmv_lanes(Ctx *ctx, const Csr *A, bool f32);
int ensure_dinv(Csr *A);
// build the symmetric storage of A's current values for FP64 or FP32 SpMVs
// when the format is requested and the values are symmetric, or the general
// grid storage when the grid format is requested and they are not (setup
// path: may allocate and synchronise; never called during stream capture)
int ensure_sym(Csr *A, bool f32);

// ------------------------------------------------------------ errors --

int set_err(Ctx *ctx, int status, const char *fmt, ...);

#define FS_CUDA_TRY(ctx, call)                                                   \
	do {                                                                         \
		cudaError_t _e = (call);                                                 \
		if (_e != cudaSuccess)                                                   \
			return ::fsg::set_err((ctx), _e == cudaErrorMemoryAllocation         \
			                                 ? FS_ERR_OUT_OF_MEMORY               \
			                                 : FS_ERR_CUDA,                      \
			                      "%s failed: %s (%s:%d)", #call,                \
			                      cudaGetErrorString(_e), __FILE__, __LINE__);   \
	} while (0)

#define FS_TRY(...)                   \
	do {                              \
		int _s = (__VA_ARGS__);       \
		if (_s != FS_OK)              \
			return _s;                \
	} while (0)

int check_launch(Ctx *ctx, const char *what);

// The calls that need stored rows, columns or values refuse a matrix-free
// operator
inline int reject_matrix_free(const Csr *A, const char *what) {
	return stores_no_rows(A)
	           ? set_err(A->ctx, FS_ERR_INVALID_ARG,
	                     "%s: not available for a matrix-free or shell operator", what)
	           : FS_OK;
}

// y = A x for a shell operator: the caller's callback, with the context's
// stream ordered before and after it (a callback may use the legacy stream
// or its own)
int shell_apply(const Csr *A, Vec *x, Vec *y);

// Programmatic dependent launch: a kernel launched with launch_pdl may be
// scheduled while the previous kernel on the stream is still finishing (its
// launch and ramp-up overlap that kernel's tail).  Such a kernel calls
// pdl_wait() first, which returns once the previous kernel has completed and
// its writes are visible, and pdl_trigger() to let the next kernel be
// scheduled early in turn.  In a kernel launched normally both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
	asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

template<class... KArgs, class... Args>
inline cudaError_t launch_pdl(cudaStream_t stream, void (*kern)(KArgs...), int grid, int block,
                              size_t smem, Args... args) {
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = dim3((unsigned)grid);
	cfg.blockDim = dim3((unsigned)block);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kern, (KArgs)args...);
}

// check_launch for a launch that returned its status
inline int check_launch_rc(Ctx *ctx, cudaError_t e, const char *what) {
	if (e != cudaSuccess) {
		ctx->launches++;
		cudaGetLastError();
		return set_err(ctx, FS_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
	}
	return check_launch(ctx, what);
}

inline bool ok_ctx(const Ctx *c) { return c && c->magic == kMagicCtx; }

// Setup copies and memsets go through the legacy default stream; a pageable
// host-to-device copy may still be in flight when cudaMemcpy returns, and the
// context's stream is non-blocking, so setup paths fence the legacy stream
// before the context's stream reads what they wrote.
inline cudaError_t fence_setup_copies() { return cudaStreamSynchronize(cudaStreamLegacy); }
inline bool ok_vec(const Vec *v) { return v && v->magic == kMagicVec && ok_ctx(v->ctx); }
inline bool ok_csr(const Csr *a) { return a && a->magic == kMagicCsr && ok_ctx(a->ctx); }

int grid_for(Ctx *ctx, int64_t n, int threads, int per_thread);

// --------------------------------------------- device helper routines --

// Error-free transforms for compensated single-precision sums
// (Ogita, Rump, Oishi, "Accurate sum and dot product", SISC 2005).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
	s = __fadd_rn(a, b);
	float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
	p = __fmul_rn(a, b);
	e = __fmaf_rn(a, b, -p);
}

// compensated accumulator: value = hi + lo
struct cf32 {
	float hi, lo;
	__device__ __forceinline__ void add(float v) {
		float s, e;
		two_sum(hi, v, s, e);
		hi = s;
		lo = __fadd_rn(lo, e);
	}
	__device__ __forceinline__ void add_prod(float a, float b) {
		float p, pe, s, se;
		two_prod(a, b, p, pe);
		two_sum(hi, p, s, se);
		hi = s;
		lo = __fadd_rn(lo, __fadd_rn(pe, se));
	}
	__device__ __forceinline__ void merge(cf32 o) {
		float s, e;
		two_sum(hi, o.hi, s, e);
		hi = s;
		lo = __fadd_rn(__fadd_rn(lo, o.lo), e);
	}
};

// Fixed-order block sum of NV doubles per thread (warp butterfly-free tree:
// shuffle-down by 16, 8, 4, 2, 1 then warp 0 sums the warp results in warp
// order).  Result valid in thread 0.  `sh` needs NV * 32 doubles.
template<int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *sh) {
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for (int k = 0; k < NV; ++k)
#pragma unroll
		for (int o = 16; o > 0; o >>= 1)
			v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
	__syncthreads();
	if (lane == 0)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			sh[k * 32 + wid] = v[k];
	__syncthreads();
	if (wid == 0) {
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			double t = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
			for (int o = 16; o > 0; o >>= 1)
				t += __shfl_down_sync(0xffffffffu, t, o);
			v[k] = t;
		}
	}
}

template<int NV>
__device__ __forceinline__ void block_sum_cf(cf32 (&v)[NV], float *sh) {
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for (int k = 0; k < NV; ++k)
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			cf32 t;
			t.hi = __shfl_down_sync(0xffffffffu, v[k].hi, o);
			t.lo = __shfl_down_sync(0xffffffffu, v[k].lo, o);
			v[k].merge(t);
		}
	__syncthreads();
	if (lane == 0)
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			sh[(2 * k) * 32 + wid] = v[k].hi;
			sh[(2 * k + 1) * 32 + wid] = v[k].lo;
		}
	__syncthreads();
	if (wid == 0) {
#pragma unroll
		for (int k = 0; k < NV; ++k) {
			cf32 t{0.f, 0.f};
			if (lane < nw) {
				t.hi = sh[(2 * k) * 32 + lane];
				t.lo = sh[(2 * k + 1) * 32 + lane];
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				cf32 u;
				u.hi = __shfl_down_sync(0xffffffffu, t.hi, o);
				u.lo = __shfl_down_sync(0xffffffffu, t.lo, o);
				t.merge(u);
			}
			v[k] = t;
		}
	}
}

// Last-block completion: every block stores its partials, fences, and bumps
// `counter`; the block that sees count == gridDim.x - 1 is the last one and
// may read all partials (no block ever waits on another).  Returns true in
// all threads of the last block; the caller resets the counter there.
__device__ __forceinline__ bool last_block(unsigned *counter) {
	__shared__ bool am_last;
	__threadfence();
	__syncthreads();
	if (threadIdx.x == 0) {
		unsigned prev = atomicAdd(counter, 1u);
		am_last = (prev == gridDim.x - 1);
	}
	__syncthreads();
	if (am_last)
		__threadfence();
	return am_last;
}

// Fixed-order sum of `n` partials (stride `stride`, component k) by one block:
// thread t sums t, t + bd, ... in order, then block_sum.  All threads call it.
template<int NV>
__device__ __forceinline__ void sum_partials(const double *part, int n,
                                             double (&out)[NV], double *sh) {
#pragma unroll
	for (int k = 0; k < NV; ++k)
		out[k] = 0.0;
	for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
		for (int k = 0; k < NV; ++k)
			out[k] += __ldcg(part + (size_t)i * NV + k);
	block_sum<NV>(out, sh);
}

}  // namespace fsg
