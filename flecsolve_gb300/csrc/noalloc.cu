// Allocation-free FP64 dot product.
//
// A variant of the library's deterministic reduction kernel (context.cu,
// red_f64<RD_DOT>) for callers that cannot allocate device memory: callers
// whose device memory is owned by another allocator (a framework's caching
// allocator or a fixed budget) and that must not call cudaMalloc themselves,
// callers that cannot take the implicit device synchronisation of
// cudaMalloc/cudaFree, and callers that hold only raw device pointers and a
// stream, with no fs_ctx (creating a context allocates its scratch).
//
// Its scratch -- one partial sum per CTA plus a completion counter -- lives in
// the file-scope array below, which every GPU that loads the library holds
// until the process exits.  The array caps the number of CTAs, hence n.
#include <cuda.h>
#include <mutex>

#include "fsgpu_internal.cuh"

namespace fsg {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaPerThread = 16;
constexpr int64_t kNaChunk = (int64_t)kNaThreads * kNaPerThread;  // 4096 elements per CTA
constexpr int kNaMaxBlocks = 16384;                               // partial sums
constexpr int kNaCounterSlots = 32;                               // 256 B for the counter
static_assert(kNaChunk * kNaMaxBlocks == FS_DOT_NOALLOC_MAX_N, "limit in fsgpu.h");

// [0, kNaMaxBlocks): per-CTA partial sums; [kNaMaxBlocks]: completion counter
// (stored as an unsigned in the first 4 bytes of that slot).
static __device__ __align__(256) double g_noalloc_scratch[kNaMaxBlocks + kNaCounterSlots];

// CTA b sums elements [b * kNaChunk, (b + 1) * kNaChunk): thread t takes
// t, t + 256, ... in order, then the fixed-order block tree; the last CTA to
// finish folds the partials in CTA order.  Deterministic for a given n.
__global__ void __launch_bounds__(kNaThreads)
dot_noalloc_kernel(const double *__restrict__ x, const double *__restrict__ y, int64_t n,
                   double *scratch, double *result) {
	__shared__ double sh[32];
	unsigned *counter = reinterpret_cast<unsigned *>(scratch + kNaMaxBlocks);
	const int64_t base = (int64_t)blockIdx.x * kNaChunk;
	double acc[1] = {0.0};
#pragma unroll
	for (int j = 0; j < kNaPerThread; ++j) {
		const int64_t i = base + threadIdx.x + (int64_t)j * kNaThreads;
		if (i < n)
			acc[0] = fma(x[i], y[i], acc[0]);
	}
	block_sum<1>(acc, sh);
	if (threadIdx.x == 0)
		scratch[blockIdx.x] = acc[0];
	if (last_block(counter)) {
		double r[1];
		sum_partials<1>(scratch, gridDim.x, r, sh);
		if (threadIdx.x == 0) {
			*result = r[0];
			*counter = 0;
		}
	}
}

// The scratch array's device address belongs to a CUDA context (the device's
// primary context under the runtime API, or a context the caller made
// current through the driver API): it is looked up once per context and
// cached under that context.
typedef CUresult (*ctx_get_current_fn)(CUcontext *);
std::mutex g_na_mutex;
constexpr int kNaCtxSlots = 64;
CUcontext g_na_ctx[kNaCtxSlots] = {};
double *g_na_addr[kNaCtxSlots] = {};
int g_na_used = 0;

ctx_get_current_fn ctx_get_current() {
	static ctx_get_current_fn fn = [] {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
		        cudaSuccess ||
		    q != cudaDriverEntryPointSuccess) {
			cudaGetLastError();
			p = nullptr;
		}
		return reinterpret_cast<ctx_get_current_fn>(p);
	}();
	return fn;
}

// the scratch address in the calling thread's current context (null on error)
double *scratch_address() {
	ctx_get_current_fn get = ctx_get_current();
	if (!get)
		return nullptr;
	CUcontext c = nullptr;
	if (get(&c) != CUDA_SUCCESS)
		return nullptr;
	std::lock_guard<std::mutex> lock(g_na_mutex);
	for (int i = 0; c && i < g_na_used; ++i)
		if (g_na_ctx[i] == c)
			return g_na_addr[i];
	// host code cannot use the symbol itself as a device address; the lookup
	// also makes the device's primary context current when none is
	double *p = nullptr;
	if (cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch) != cudaSuccess || !p) {
		cudaGetLastError();
		return nullptr;
	}
	if (!c && get(&c) != CUDA_SUCCESS)
		return nullptr;
	if (c && g_na_used < kNaCtxSlots) {
		g_na_ctx[g_na_used] = c;
		g_na_addr[g_na_used] = p;
		++g_na_used;
	}
	return p;
}

}  // namespace
}  // namespace fsg

using namespace fsg;

extern "C" FS_API int fs_dot_f64_noalloc(const double *x, const double *y, int64_t n,
                                         double *result, void *stream) {
	if (!result || n < 0 || (n > 0 && (!x || !y)))
		return FS_ERR_INVALID_ARG;
	if (n > FS_DOT_NOALLOC_MAX_N)
		return FS_ERR_INVALID_ARG;  // beyond the scratch array's capacity
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) {
		cudaGetLastError();
		return FS_ERR_NO_DEVICE;
	}
	double *scratch = scratch_address();
	if (!scratch)
		return FS_ERR_CUDA;
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	// the array keeps the previous call's contents: the counter must start at 0
	if (cudaMemsetAsync(scratch + kNaMaxBlocks, 0, sizeof(unsigned), st) != cudaSuccess) {
		cudaGetLastError();
		return FS_ERR_CUDA;
	}
	if (n == 0) {
		if (cudaMemsetAsync(result, 0, sizeof(double), st) != cudaSuccess) {
			cudaGetLastError();
			return FS_ERR_CUDA;
		}
		return FS_OK;
	}
	const int blocks = (int)((n + kNaChunk - 1) / kNaChunk);
	dot_noalloc_kernel<<<blocks, kNaThreads, 0, st>>>(x, y, n, scratch, result);
	if (cudaGetLastError() != cudaSuccess)
		return FS_ERR_CUDA;
	return FS_OK;
}
